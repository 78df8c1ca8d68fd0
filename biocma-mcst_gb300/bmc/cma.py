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


def turbulence_kla(energy_dissipation, liquid_volume, gas_volume, bubble_diameter: float = 5e-3) -> np.ndarray:
    """kla (1/s) of O2 per compartment under the reference's FlowmapTurbulence
    mass-transfer model (from the case's turbulent energy dissipation and the
    gas fraction; include/bmc.h bmc_mtr_turbulence_kla): the O2 column of a
    two-phase scenario's kla (scenarios.with_gas(kla=...))."""
    eps = np.ascontiguousarray(energy_dissipation, dtype=np.float64)
    vl = np.ascontiguousarray(liquid_volume, dtype=np.float64)
    vg = np.ascontiguousarray(gas_volume, dtype=np.float64)
    if not (eps.shape == vl.shape == vg.shape) or eps.ndim != 1:
        raise ValueError("one value per compartment in each array")
    out = np.zeros(len(eps))
    call("bmc_mtr_turbulence_kla", len(eps), _p(eps), _p(vl), _p(vg), float(bubble_diameter), _p(out))
    return out


def read_field(path: str) -> np.ndarray:
    """Values of a case field file (uint32 count + float64 values)."""
    n = ct.c_uint64()
    call("bmc_cma_read_field", path.encode(), 0, None, ct.byref(n))
    out = np.zeros(n.value)
    call("bmc_cma_read_field", path.encode(), n.value, _p(out), ct.byref(n))
    return out


# Entry kinds of a case descriptor (those of the reference's 0-D fixture).
KIND_LIQUID_FLOW = 0
KIND_LIQUID_VOLUME = 3


def read_case(path: str) -> dict:
    """A case descriptor (bmc_cma_read_case / bmc_cma_case_entry): the four
    header words and the float as stored, and the entries as (kind, path)
    pairs in file order."""
    words = (ct.c_uint32 * 4)()
    t0, n = ct.c_double(), ct.c_uint32()
    call("bmc_cma_read_case", path.encode(), words, ct.byref(t0), ct.byref(n))
    entries = []
    for k in range(n.value):
        kind = ct.c_uint32()
        name = ct.create_string_buffer(4096)
        call("bmc_cma_case_entry", path.encode(), k, ct.byref(kind), name, len(name))
        entries.append((kind.value, name.value.decode()))
    return {"words": list(words), "t0": t0.value, "entries": entries}


def read_flowmap(path: str):
    """A liquid flow map file (bmc_cma_read_flowmap): (rows, columns, row
    indices, column indices, flows)."""
    nr, nc, nnz = ct.c_uint32(), ct.c_uint32(), ct.c_uint64()
    call("bmc_cma_read_flowmap", path.encode(), ct.byref(nr), ct.byref(nc), ct.byref(nnz), 0, None, None, None)
    r = np.zeros(nnz.value, np.uint64)
    c = np.zeros(nnz.value, np.uint64)
    f = np.zeros(nnz.value)
    if nnz.value:
        call("bmc_cma_read_flowmap", path.encode(), ct.byref(nr), ct.byref(nc), ct.byref(nnz), nnz.value, _p(r), _p(c),
             _p(f))
    return nr.value, nc.value, r, c, f


def load_case(folder: str, descriptor: str = "cma_case") -> networks.Network:
    """The Network of a CMA case folder: the descriptor names the liquid
    volume field and the liquid flow map (paths relative to the folder); the
    map must be square over the volumes' compartments."""
    import os

    case = read_case(os.path.join(folder, descriptor))
    files = {}
    for kind, name in case["entries"]:
        files.setdefault(kind, os.path.normpath(os.path.join(folder, name)))
    if KIND_LIQUID_VOLUME not in files or KIND_LIQUID_FLOW not in files:
        raise ValueError("the case descriptor names no liquid volume field or no liquid flow map")
    vol = read_field(files[KIND_LIQUID_VOLUME])
    nr, nc, r, c, f = read_flowmap(files[KIND_LIQUID_FLOW])
    if not (nr == nc == len(vol)):
        raise ValueError(f"flow map of {nr} x {nc} over {len(vol)} compartment volumes")
    return network(vol, r, c, f)


def write_case(folder: str, volumes, rows, cols, flows, words=(1, 1, 1, 0), t0: float = 0.0) -> None:
    """Writes a case folder in the layout the readers take: cma_case naming
    ./vofL.raw (kind 3) and ./flowL.raw (kind 0), as the reference's 0-D
    fixture does, the volume field and the flow map."""
    import os
    import struct

    vol = np.ascontiguousarray(volumes, dtype="<f8")
    r = np.ascontiguousarray(rows, dtype="<u8")
    c = np.ascontiguousarray(cols, dtype="<u8")
    f = np.ascontiguousarray(flows, dtype="<f8")
    if not (len(r) == len(c) == len(f)):
        raise ValueError("rows, cols and flows differ in length")
    os.makedirs(folder, exist_ok=True)
    desc = struct.pack("<4Id", *words, t0) + struct.pack("<Q", 2)
    for kind, name in ((KIND_LIQUID_VOLUME, b"./vofL.raw"), (KIND_LIQUID_FLOW, b"./flowL.raw")):
        desc += struct.pack("<BI", kind, len(name)) + name
    with open(os.path.join(folder, "cma_case"), "wb") as fh:
        fh.write(desc)
    with open(os.path.join(folder, "vofL.raw"), "wb") as fh:
        fh.write(struct.pack("<I", len(vol)) + vol.tobytes())
    n = len(vol)
    with open(os.path.join(folder, "flowL.raw"), "wb") as fh:
        fh.write(struct.pack("<II", n, n))
        for a in (r, c, f):
            fh.write(struct.pack("<Q", len(a)) + a.tobytes())


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
