"""Writes the golden fixtures of tests/golden/ (run from the repository root).

Every value here is typed in from a published source or worked by hand from
the reference's source code; nothing is computed by this repository's code:

* philox_kat.json -- Philox4x32-10 known-answer vectors published with
  Random123 (Salmon et al., SC'11; kat_vectors file of the Random123
  distribution): counter, key, output.
* move_cases.json -- next-compartment outcomes of the reference bisection
  (apps/libs/simulation/public/simulation/kernels/move_kernel.hpp L89-L101:
  left=0, right=K-1; while left<right: mid=(left+right)>>1; left=mid+1 if
  u > CDF[mid] else right=mid), worked by hand for a 3-neighbour row, and the
  leave decision of probability_leaving<fast_tag> (probability_leaving.hpp
  L234: dt*flow/volume > u).
* container_counts.json -- the counts asserted by the reference's container
  test (apps/libs/mc/tests/test_container.cpp L14-L127): 1000 particles,
  10 divisions -> 1010 after merge; 10 removed -> 990; capacity =
  n * allocation_factor.
* cma_cases.json -- the transition matrices of the reference's (disabled)
  CmaUtils test (apps/libs/cma_utils/tests/test_transition_matrix.cpp
  L7-L25), the cumulative probabilities of the 3x3 case worked by hand from
  P(I_j | L) = F(i, j) / sum_k F(i, k) (documentation/pages/03_cma.md), and
  the bytes of the two field files of the reference's 0-D case fixture
  (apps/api/tests/data/0d/vofL.raw and turbE.raw.raw, 12 bytes each: uint32
  count 1, then float64 0.02 and 0.5), and the bytes of the same fixture's
  case descriptor (cma_case, 63 bytes) and liquid flow map (flowL.raw, 32
  bytes), typed in from the fixture with the fields they hold.
"""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    philox = [
        {"ctr": [0, 0, 0, 0], "key": [0, 0],
         "out": [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]},
        {"ctr": [0xFFFFFFFF] * 4, "key": [0xFFFFFFFF, 0xFFFFFFFF],
         "out": [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]},
        {"ctr": [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], "key": [0xA4093822, 0x299F31D0],
         "out": [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]},
    ]
    # row CDF [0.2, 0.5, 1.0] with neighbours [7, 3, 9]
    move = {
        "cdf": [0.2, 0.5, 1.0],
        "neighbors": [7, 3, 9],
        "cases": [
            {"u": 0.1, "next": 7}, {"u": 0.2, "next": 7}, {"u": 0.25, "next": 3},
            {"u": 0.5, "next": 3}, {"u": 0.75, "next": 9}, {"u": 0.9999999, "next": 9},
        ],
        # K = 4 with a padded last slot (CDF 1.0, neighbour repeated)
        "cdf4": [0.25, 0.5, 0.999999999, 1.0],
        "neighbors4": [1, 2, 3, 3],
        "cases4": [{"u": 0.125, "next": 1}, {"u": 0.375, "next": 2},
                   {"u": 0.9999999999, "next": 3}, {"u": 0.5, "next": 2}],
        # leave iff dt*Q/V > u
        "leave": [
            {"dt": 0.1, "q": 1e-3, "v": 1e-3, "u": 0.0999, "leave": True},
            {"dt": 0.1, "q": 1e-3, "v": 1e-3, "u": 0.1001, "leave": False},
            {"dt": 0.05, "q": 2e-3, "v": 4e-3, "u": 0.02, "leave": True},
        ],
    }
    container = {"size": 1000, "ndiv": 10, "after_merge": 1010, "to_remove": 10,
                 "after_remove": 990, "allocation_factor_cuda": 1.5, "allocation_factor_cpu": 2.5}
    cma = {
        "transition": [
            {"flows": [[1, 2], [3, 4]], "expected": [[-2, 2], [3, -3]]},
            {"flows": [[1, 2, 3], [4, 5, 6], [7, 8, 9]], "expected": [[-5, 2, 3], [4, -10, 6], [7, 8, -15]]},
        ],
        # 3x3 case: row 0 -> {1: 2, 2: 3}, row 1 -> {0: 4, 2: 6}, row 2 -> {0: 7, 1: 8}
        "derive_3x3": {"K": 2, "neighbors": [[1, 2], [0, 2], [0, 1]], "out_flow": [5, 10, 15],
                       "cdf": [[0.4, 1.0], [0.4, 1.0], [7 / 15, 1.0]]},
        "fields_0d": [
            {"file": "vofL.raw", "hex": "010000007b14ae47e17a943f", "values": [0.02]},
            {"file": "turbE.raw.raw", "hex": "01000000000000000000e03f", "values": [0.5]},
        ],
        # the fixture's descriptor: words 1, 1, 1, 0; float 0.0; two entries
        # (kind 3 "./vofL.raw", kind 0 "./flowL.raw"); its flow map: 1 x 1
        # with three zero uint64 words after the dimensions
        "case_0d": {
            "cma_case": "01000000" "01000000" "01000000" "00000000" "0000000000000000" "0200000000000000"
                        "03" "0a000000" + b"./vofL.raw".hex() + "00" "0b000000" + b"./flowL.raw".hex(),
            "flowL.raw": "01000000" "01000000" + "00" * 24,
            "words": [1, 1, 1, 0], "t0": 0.0,
            "entries": [[3, "./vofL.raw"], [0, "./flowL.raw"]],
            "n_rows": 1, "n_cols": 1, "nnz": 0, "volume": [0.02],
        },
    }
    for name, obj in (("philox_kat.json", philox), ("move_cases.json", move),
                      ("container_counts.json", container), ("cma_cases.json", cma)):
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(obj, f, indent=1)


if __name__ == "__main__":
    main()
