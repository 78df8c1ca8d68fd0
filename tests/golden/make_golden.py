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
    for name, obj in (("philox_kat.json", philox), ("move_cases.json", move),
                      ("container_counts.json", container)):
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(obj, f, indent=1)


if __name__ == "__main__":
    main()
