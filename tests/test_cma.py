"""CMA ingestion: flow map -> neighbours, out-flows, cumulative probabilities,
liquid transition; automatic time step; case field files.

libbmc's host functions (no device work) are checked against the known
answers of the reference's CmaUtils test and 0-D case fixture
(tests/golden/cma_cases.json, written by tests/golden/make_golden.py), and
bit for bit against the Python derivation the seeded generators use; the GPU
test runs a scenario whose domain came through the C-ABI derivation against
the CPU restatement.
"""
import json
import os

import numpy as np
import pytest

from bmc import cma, networks, scenarios
from bmc._lib import BmcError

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cma_cases.json")


def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def dense_coo(F):
    F = np.asarray(F, dtype=np.float64)
    r, c = np.nonzero(np.ones_like(F))
    return r, c, F[r, c]


@pytest.mark.parametrize("case", range(2))
def test_transition_known_answers(case):
    g = golden()["transition"][case]
    n = len(g["flows"])
    tr, tc, tv = cma.transition(n, *dense_coo(g["flows"]))
    T = np.zeros((n, n))
    T[tr.astype(int), tc.astype(int)] = tv
    assert np.array_equal(T, np.array(g["expected"], dtype=np.float64))
    # sorted by (row, col), diagonal included once per compartment
    key = tr * n + tc
    assert np.all(np.diff(key.astype(np.int64)) > 0)


def test_derive_known_answer():
    g = golden()["derive_3x3"]
    d = cma.derive(3, *dense_coo(golden()["transition"][1]["flows"]))
    assert d["K"] == g["K"]
    assert np.array_equal(d["neighbors"], np.array(g["neighbors"], dtype=np.uint64))
    assert np.array_equal(d["out_flow"], np.array(g["out_flow"], dtype=np.float64))
    assert np.array_equal(d["cdf"], np.array(g["cdf"], dtype=np.float64))


def test_field_files_of_the_0d_case(tmp_path):
    for fx in golden()["fields_0d"]:
        p = tmp_path / fx["file"]
        p.write_bytes(bytes.fromhex(fx["hex"]))
        assert np.array_equal(cma.read_field(str(p)), np.array(fx["values"]))
    bad = tmp_path / "short.raw"
    bad.write_bytes(bytes.fromhex("02000000000000000000e03f"))  # count 2, one value
    with pytest.raises(BmcError, match="size"):
        cma.read_field(str(bad))
    with pytest.raises(BmcError, match="cannot open"):
        cma.read_field(str(tmp_path / "missing.raw"))


def write_fixture_case(folder):
    g = golden()
    c0 = g["case_0d"]
    (folder / "cma_case").write_bytes(bytes.fromhex(c0["cma_case"]))
    (folder / "flowL.raw").write_bytes(bytes.fromhex(c0["flowL.raw"]))
    (folder / "vofL.raw").write_bytes(bytes.fromhex(g["fields_0d"][0]["hex"]))
    return c0


def test_case_descriptor_and_flow_map_of_the_0d_case(tmp_path):
    """The reference's 0-D case: the descriptor's words, float and entries,
    and its 1 x 1 flow map with no flow."""
    c0 = write_fixture_case(tmp_path)
    case = cma.read_case(str(tmp_path / "cma_case"))
    assert case["words"] == c0["words"] and case["t0"] == c0["t0"]
    assert [list(e) for e in case["entries"]] == c0["entries"]
    nr, nc, r, c, f = cma.read_flowmap(str(tmp_path / "flowL.raw"))
    assert (nr, nc, len(r)) == (c0["n_rows"], c0["n_cols"], c0["nnz"])
    net = cma.load_case(str(tmp_path))
    assert net.n_c == 1 and net.volume.tolist() == c0["volume"]
    assert net.out_flow.tolist() == [0.0] and net.neighbors.ravel().tolist() == [0]


def test_written_case_reads_back(tmp_path):
    """A case written in the readers' layout loads into the Network the
    flow map gives directly (bit for bit)."""
    net0 = networks.lattice_vortex(4, seed=5)
    cma.write_case(str(tmp_path), net0.volume, net0.src, net0.dst, net0.flow)
    net = cma.load_case(str(tmp_path))
    ref = cma.network(net0.volume, net0.src, net0.dst, net0.flow)
    for k in ("volume", "neighbors", "out_flow", "cdf", "in_ptr", "in_idx", "in_flow"):
        assert np.array_equal(np.asarray(getattr(net, k)).view(np.uint8), np.asarray(getattr(ref, k)).view(np.uint8)), k
    # the descriptor the writer makes has the fixture's header and entries
    c0 = golden()["case_0d"]
    assert bytes.fromhex(c0["cma_case"]) == (tmp_path / "cma_case").read_bytes()


@pytest.mark.parametrize("what,msg", [
    ("case_short", "shorter"), ("case_tail", "after its last entry"), ("case_count", "entry count"),
    ("case_path", "past the end"), ("flow_short", "shorter"), ("flow_size", "size differs"),
    ("flow_lengths", "differ in length"), ("flow_range", "outside"),
])
def test_malformed_case_files_are_refused(tmp_path, what, msg):
    import struct

    c0 = golden()["case_0d"]
    case = bytes.fromhex(c0["cma_case"])
    flow = struct.pack("<II", 2, 2) + struct.pack("<Q", 1) + struct.pack("<Q", 0) + struct.pack("<Q", 1) + \
        struct.pack("<Q", 1) + struct.pack("<Q", 1) + struct.pack("<d", 1e-3)
    bad = {
        "case_short": case[:20], "case_tail": case + b"\0", "case_count": case[:24] + struct.pack("<Q", 99) + case[32:],
        "case_path": case[:-3], "flow_short": flow[:20], "flow_size": flow + b"\0" * 8,
        "flow_lengths": struct.pack("<II", 2, 2) + struct.pack("<Q", 1) + struct.pack("<Q", 0) + struct.pack("<Q", 0) +
        struct.pack("<Q", 1) + struct.pack("<d", 1e-3),
        "flow_range": struct.pack("<II", 2, 2) + struct.pack("<Q", 1) + struct.pack("<Q", 2) + struct.pack("<Q", 1) +
        struct.pack("<Q", 1) + struct.pack("<Q", 1) + struct.pack("<d", 1e-3),
    }[what]
    p = tmp_path / "file"
    p.write_bytes(bad)
    with pytest.raises(BmcError, match=msg):
        if what.startswith("case"):
            cma.read_case(str(p))
        else:
            cma.read_flowmap(str(p))
    # the well-formed two-compartment map of this test reads
    p.write_bytes(flow)
    nr, nc, r, c, f = cma.read_flowmap(str(p))
    assert (nr, nc, r.tolist(), c.tolist(), f.tolist()) == (2, 2, [0], [1], [1e-3])


@pytest.mark.parametrize("net", [networks.lattice_vortex(8, seed=3), networks.lattice_vortex(4, seed=9),
                                 networks.ring_network(10, 2, seed=42, max_courant=0.5, dt=0.1)],
                         ids=["lattice8", "lattice4", "ring10"])
def test_derivation_matches_the_generators(net):
    """The C-ABI derivation reproduces the generators' arrays bit for bit."""
    d = cma.derive(net.n_c, net.src, net.dst, net.flow)
    assert d["K"] == net.K
    assert np.array_equal(d["neighbors"], net.neighbors.astype(np.uint64))
    assert np.array_equal(d["out_flow"].view(np.uint64), net.out_flow.view(np.uint64))
    assert np.array_equal(d["cdf"].view(np.uint64), net.cdf.view(np.uint64))
    assert np.all(d["cdf"][:, -1] == 1.0)
    tr, tc, tv = cma.transition(net.n_c, net.src, net.dst, net.flow)
    T = np.zeros((net.n_c, net.n_c))
    T[tr.astype(int), tc.astype(int)] = tv
    assert np.array_equal(T, net.transition_dense())


def test_self_zero_and_duplicate_flows():
    rows = [0, 0, 0, 1, 1, 2, 0]
    cols = [0, 1, 2, 2, 1, 0, 1]
    flows = [9.0, 1.0, 0.0, 2.0, 5.0, 3.0, 0.5]  # (0,0) and (1,1) self, (0,2) zero, (0,1) twice
    d = cma.derive(3, rows, cols, flows)
    assert d["K"] == 1
    assert d["neighbors"].ravel().tolist() == [1, 2, 0]
    assert d["out_flow"].tolist() == [1.5, 2.0, 3.0]
    assert d["cdf"].ravel().tolist() == [1.0, 1.0, 1.0]
    tr, tc, tv = cma.transition(3, rows, cols, flows)
    assert list(zip(tr.tolist(), tc.tolist(), tv.tolist())) == [
        (0, 0, -1.5), (0, 1, 1.5), (1, 1, -2.0), (1, 2, 2.0), (2, 0, 3.0), (2, 2, -3.0)]
    # a compartment without out-flow: itself as neighbour, probability 1
    d = cma.derive(3, [0], [1], [1.0])
    assert d["neighbors"].ravel().tolist() == [1, 1, 2]
    assert d["out_flow"].tolist() == [1.0, 0.0, 0.0]


@pytest.mark.parametrize("rows,cols,flows,msg", [
    ([0], [3], [1.0], "out of range"),
    ([0], [1], [-1.0], ">= 0"),
    ([0], [1], [np.nan], "finite"),
])
def test_bad_flow_maps_are_refused(rows, cols, flows, msg):
    with pytest.raises(BmcError, match=msg):
        cma.derive(3, rows, cols, flows)
    with pytest.raises(BmcError, match=msg):
        cma.transition(3, rows, cols, flows)


def test_time_step():
    v = np.array([[1e-3, 2e-3, 0.0], [1e-3, 1e-3, 1e-3]])
    q = np.array([[4e-5, 2e-5, 7.0], [3e-5, 5e-5, 6e-5]])
    # min over maps and compartments of positive volume: 2e-5 / 2e-3 = 1e-2
    assert cma.time_step(v, q) == (2e-5 / 2e-3) / 100.0
    assert cma.time_step(v, q, user_dt=0.25) == 0.25
    with pytest.raises(BmcError, match="impossible"):
        cma.time_step(np.zeros((1, 3)), q[:1])
    with pytest.raises(BmcError, match="impossible"):
        cma.time_step(v[1:], np.zeros((1, 3)))


def test_network_from_a_flow_map():
    net0 = networks.lattice_vortex(4, seed=5)
    net = cma.network(net0.volume, net0.src, net0.dst, net0.flow)
    for k in ("neighbors", "out_flow", "cdf", "in_ptr", "in_idx", "in_flow"):
        assert np.array_equal(getattr(net, k), getattr(net0, k)), k
    assert net.K == net0.K


@pytest.mark.gpu
def test_gpu_domain_from_a_flow_map(oracle_mod):
    """A scenario whose domain and transition come through bmc_cma_derive /
    bmc_cma_transition steps like the CPU restatement, bit for bit."""
    from test_gpu_parity import assert_same_liquid, assert_same_particles, assert_same_stats, make_pair

    from bmc.sim import GpuScenario

    sc = scenarios.workload(2, n_particles=50000)
    F = sc.net
    sc.net = cma.network(F.volume, F.src, F.dst, F.flow)
    # and through a case folder written and read back (bmc_cma_read_case,
    # bmc_cma_read_field, bmc_cma_read_flowmap)
    import tempfile

    with tempfile.TemporaryDirectory() as d:
        cma.write_case(d, F.volume, F.src, F.dst, F.flow)
        from_case = cma.load_case(d)
    for k in ("neighbors", "out_flow", "cdf", "in_ptr", "in_idx", "in_flow"):
        assert np.array_equal(getattr(from_case, k), getattr(sc.net, k)), k
    sc.net = from_case
    g, o = make_pair(oracle_mod, sc)
    # the same flow map installed again through the C-ABI on a second scenario
    g2 = GpuScenario(sc)  # same seed: the same initial particles and weight
    cma.install(g2, F.volume, F.src, F.dst, F.flow)
    assert g2.weight == g.weight
    for k in range(5):
        gs, os_ = g.step(), o.step()
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
        gs2 = g2.step()
        assert_same_stats(gs2, os_, f"installed, step {k}")
        assert_same_liquid(g2, o, f"installed, step {k}")
    assert_same_particles(g, o, "end")
    assert_same_particles(g2, o, "installed, end")
