"""CMA ingestion through libbmc's host functions (include/bmc.h, "CMA
ingestion"): the per-compartment arrays and the liquid transition derived
from a flow map F(i, j), the automatic time step of a set of flow maps, and
the field files of a CMA case.  Nothing here runs on the device.

The reference obtains these from rcmtool (outside its tree) through
CmaUtils; the derivations follow documentation/pages/03_cma.md and are
pinned by the known answers of
apps/libs/cma_utils/tests/test_transition_matrix.cpp L7-L25.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import networks
from ._lib import call


def _p(a: np.ndarray):
    return a.ctypes.data if a.size else None


def _coo(rows, cols, flows):
    r = np.ascontiguousarray(rows, dtype=np.uint64)
    c = np.ascontiguousarray(cols, dtype=np.uint64)
    f = np.ascontiguousarray(flows, dtype=np.float64)
    if not (r.shape == c.shape == f.shape and r.ndim == 1):
        raise ValueError("rows, cols and flows must be 1-D arrays of one length")
    return r, c, f


def derive(n_c: int, rows, cols, flows) -> dict:
    """Neighbours [n_c, K] (uint64), out-flows [n_c], cumulative destination
    probabilities [n_c, K] of a flow map given as COO triplets."""
    r, c, f = _coo(rows, cols, flows)
    K = ct.c_uint32()
    call("bmc_cma_derive", n_c, len(f), _p(r), _p(c), _p(f), ct.byref(K), 0, None, None, None)
    k = K.value
    nbr = np.zeros((n_c, k), dtype=np.uint64)
    outf = np.zeros(n_c)
    cdf = np.zeros((n_c, k))
    call("bmc_cma_derive", n_c, len(f), _p(r), _p(c), _p(f), ct.byref(K), k, _p(nbr), _p(outf), _p(cdf))
    return {"K": k, "neighbors": nbr, "out_flow": outf, "cdf": cdf}


def transition(n_c: int, rows, cols, flows):
    """Liquid transition matrix in COO form (rows, cols, values), sorted by
    (row, col): F(i, j) off the diagonal, minus the out-flow on it."""
    r, c, f = _coo(rows, cols, flows)
    nnz = ct.c_uint64()
    call("bmc_cma_transition", n_c, len(f), _p(r), _p(c), _p(f), ct.byref(nnz), 0, None, None, None)
    n = nnz.value
    tr, tc, tv = np.zeros(n, np.uint64), np.zeros(n, np.uint64), np.zeros(n)
    call("bmc_cma_transition", n_c, len(f), _p(r), _p(c), _p(f), ct.byref(nnz), n, _p(tr), _p(tc), _p(tv))
    return tr, tc, tv


def time_step(volumes, out_flows, user_dt: float = 0.0) -> float:
    """The run's time step: user_dt when positive, else min(out-flow / volume)
    over every flow map and compartment of positive volume, / 100."""
    v = np.ascontiguousarray(np.atleast_2d(volumes), dtype=np.float64)
    q = np.ascontiguousarray(np.atleast_2d(out_flows), dtype=np.float64)
    if v.shape != q.shape:
        raise ValueError("volumes and out_flows must have one shape")
    dt = ct.c_double()
    call("bmc_cma_time_step", float(user_dt), v.shape[0], v.shape[1], _p(v), _p(q), ct.byref(dt))
    return dt.value


def read_field(path: str) -> np.ndarray:
    """Values of a case field file (uint32 count + float64 values)."""
    n = ct.c_uint64()
    call("bmc_cma_read_field", path.encode(), 0, None, ct.byref(n))
    out = np.zeros(n.value)
    call("bmc_cma_read_field", path.encode(), n.value, _p(out), ct.byref(n))
    return out


def network(volume, rows, cols, flows) -> networks.Network:
    """A Network (the form scenarios carry) from a flow map: the merged
    links of the derived transition, with neighbours, out-flows and
    probabilities from bmc_cma_derive."""
    vol = np.ascontiguousarray(volume, dtype=np.float64)
    n_c = len(vol)
    tr, tc, tv = transition(n_c, rows, cols, flows)
    off = tr != tc
    net = networks.Network(n_c, vol, tr[off].astype(np.int64), tc[off].astype(np.int64), tv[off].copy(),
                           meta={"source": "flow map"})
    net.finalize()
    d = derive(n_c, rows, cols, flows)
    net.K, net.neighbors, net.out_flow, net.cdf = d["K"], d["neighbors"].astype(np.uint32), d["out_flow"], d["cdf"]
    return net


def install(g, volume, rows, cols, flows) -> None:
    """Replace a GpuScenario's domain and liquid transition with those derived
    from a flow map (bmc_cma_derive + bmc_domain_update, bmc_cma_transition +
    bmc_set_transition_coo)."""
    vol = np.ascontiguousarray(volume, dtype=np.float64)
    n_c = len(vol)
    d = derive(n_c, rows, cols, flows)
    call("bmc_domain_update", g.handle, n_c, d["K"], _p(vol), _p(d["neighbors"]), _p(d["out_flow"]), _p(d["cdf"]))
    tr, tc, tv = transition(n_c, rows, cols, flows)
    call("bmc_set_transition_coo", g.handle, n_c, len(tv), _p(tr), _p(tc), _p(tv))
