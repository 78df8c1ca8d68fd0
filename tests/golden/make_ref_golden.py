"""Writes tests/golden/ref_pins.json from the reference's own code.

The reference's per-particle functions are compiled from its headers,
unmodified, against a Kokkos stand-in (oracle/refbuild/, output
oracle/_ref/libbmc_ref.so; `make -C oracle/refbuild REF=<reference tree>`).
This script calls them on seeded random and edge inputs and records inputs
and outputs; tests/test_ref_pins.py checks the oracle's functions against
the records bit for bit.  Run from the repository root:

    python tests/golden/make_ref_golden.py [<reference tree>]

Functions recorded (paths relative to the BioCMA-MCST tree):
* find_next: __find_next_compartment
  (apps/libs/simulation/public/simulation/kernels/move_kernel.hpp L62-L103)
* move: MoveFunctor::handle_move (move_kernel.hpp L393-L437) with
  probability_leaving<fast_tag> (probability_leaving.hpp L35-L48)
* leave: MoveFunctor::operator()(TagLeave) + handle_exit (move_kernel.hpp
  L348-L359, L588-L648) with probability_leaving<precision_tag> (L18-L33),
  including the draws on each side of every exit boundary
* fixed_length_update / fixed_length_division (fixed_length.hpp L123-L161)
* simple_acetate_update / _division / _init (simple_acetate.hpp L129-L250)
* erfinv_f / erfinv_d / norminv_f / truncnorm_f (prng_extension.hpp
  L82-L147 and TruncatedNormal::draw_from)
* check_div (apps/libs/models/public/models/utils.hpp L64-L69)
* feed_flow: FeedDescriptor::update (apps/libs/simulation/src/
  feed_descriptor.cpp L12-L36) of Linear and Exponential feeds at relative
  times accumulated by SimulatimeTimes::advance (simulation_times.hpp L15-L18)

Floats are stored as their IEEE bit patterns (uint32 / uint64) so the file
round-trips exactly.
"""
import ctypes as ct
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "libbmc_ref.so")

F32, F64, U64, I32, U32 = ct.c_float, ct.c_double, ct.c_uint64, ct.c_int32, ct.c_uint32
PF, PD, PU64, PI32 = (ct.POINTER(t) for t in (F32, F64, U64, I32))


def b32(x) -> int:
    return int(np.float32(x).view(np.uint32))


def b64(x) -> int:
    return int(np.float64(x).view(np.uint64))


def load(ref_root: str):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "refbuild"), f"REF={ref_root}"], check=True)
    L = ct.CDLL(LIB)
    sig = {
        "ref_find_next": (U64, [I32, U32, U32, PU64, PD, U64, F64]),
        "ref_handle_move": (U64, [U32, U32, PD, PD, PU64, PD, F64, U64, F32, F32, PU64]),
        "ref_leave_one": (U64, [U32, PU64, PD, PD, F64, U64, I32, F32, F32, PI32, PF]),
        "ref_leave_precise": (I32, [F32, F64, F64, F64]),
        "ref_fixed_length_update": (I32, [F32, PF, F64, PF]),
        "ref_fixed_length_division": (None, [PF, PF]),
        "ref_simple_acetate_update": (I32, [F32, PF, F64, F64, PF]),
        "ref_simple_acetate_division": (None, [PF, PF, PD, I32]),
        "ref_simple_acetate_init": (None, [PF, PD, I32]),
        "ref_erfinv_f": (F32, [F32]),
        "ref_erfinv_d": (F64, [F64]),
        "ref_norminv_f": (F32, [F32, F32, F32]),
        "ref_truncnorm_f": (F32, [F64, F32, F32, F32, F32]),
        "ref_check_div_f": (I32, [F32, F32]),
        "ref_feed_flow": (F64, [I32, F64, F64, F64, F64]),
        "ref_relative_time": (F64, [F64, U32]),
        "ref_assert_failures": (ct.c_long, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def ptr(a, t):
    return a.ctypes.data_as(t)


def draw_value(k: int) -> float:
    """The k-th value of the draw source: (2k + 1) / 2^24 (exact in float)."""
    return (2.0 * k + 1.0) / 16777216.0


def cdf_row(rng, K: int):
    kind = rng.integers(4)
    w = rng.lognormal(0.0, 1.0, size=K)
    if kind == 1 and K > 1:
        w[rng.integers(K)] = 0.0  # a zero-probability neighbour (repeated CDF value)
    c = np.cumsum(w) / w.sum()
    c[-1] = 1.0
    if kind == 2:
        c[-1] = 0.999999999  # a last entry just below one
    return c


def u_cases(rng, row):
    us = [0.0, 1.0]
    for v in row:
        us += [float(v), float(np.nextafter(v, 0.0)), float(np.nextafter(v, 2.0))]
        us.append(float(np.float32(v)))  # the float draw nearest the entry
    us += [draw_value(int(k)) for k in rng.integers(0, 1 << 23, size=6)]
    return [u for u in us if 0.0 <= u <= 1.0]


def gen_find_next(L, rng):
    out = []
    for _ in range(40):
        K = int(rng.integers(1, 10))
        n_c = 3
        cdf = np.stack([cdf_row(rng, K) for _ in range(n_c)])
        nbr = rng.integers(0, 50, size=(n_c, K)).astype(np.uint64)
        for i in range(n_c):
            cases = []
            for u in u_cases(rng, cdf[i]):
                for search in (1, 0):
                    r = L.ref_find_next(search, n_c, K, ptr(nbr, PU64), ptr(cdf, PD), i, u)
                    cases.append([b64(u), search, int(r)])
            out.append({"K": K, "i": i, "cdf": [b64(v) for v in cdf[i]], "nbr": [int(v) for v in nbr[i]],
                        "cases": cases})
    return out


def gen_move(L, rng):
    out = []
    for _ in range(60):
        n_c, K = 5, int(rng.integers(1, 8))
        vol = rng.uniform(1e-4, 2e-3, size=n_c)
        diag = rng.uniform(0.0, 1e-2, size=n_c) * vol
        cdf = np.stack([cdf_row(rng, K) for _ in range(n_c)])
        nbr = rng.integers(0, n_c, size=(n_c, K)).astype(np.uint64)
        dt = float(rng.uniform(0.01, 0.5))
        cases = []
        for _ in range(40):
            pos = int(rng.integers(n_c))
            p_move = dt * diag[pos] / vol[pos]
            if rng.random() < 0.5:  # draws at the leave boundary
                k0 = int(np.floor((p_move * 16777216.0 - 1.0) / 2.0))
                k = min(max(k0 + int(rng.integers(-2, 3)), 0), (1 << 23) - 1)
            else:
                k = int(rng.integers(0, 1 << 23))
            u1 = draw_value(k)
            u2 = draw_value(int(rng.integers(0, 1 << 23)))
            if rng.random() < 0.3:
                u2 = float(np.float32(cdf[pos, int(rng.integers(K))]))
            moved = U64(0)
            r = L.ref_handle_move(n_c, K, ptr(vol, PD), ptr(diag, PD), ptr(nbr, PU64), ptr(cdf, PD), dt, pos,
                                  u1, u2, ct.byref(moved))
            cases.append({"pos": pos, "u1": b32(u1), "u2": b32(u2), "next": int(r), "moved": int(moved.value)})
        out.append({"n_c": n_c, "K": K, "dt": b64(dt), "volume": [b64(v) for v in vol],
                    "diag": [b64(v) for v in diag], "cdf": [b64(v) for v in cdf.ravel()],
                    "nbr": [int(v) for v in nbr.ravel()], "cases": cases})
    return out


def exit_boundary(L, dt, F, V):
    """Smallest k whose draw exits (bisection over the reference's own test,
    monotone in the draw); 2^23 when no draw exits."""
    lo, hi = 0, 1 << 23
    while lo < hi:
        mid = (lo + hi) // 2
        if L.ref_leave_precise(draw_value(mid), V, F, dt):
            hi = mid
        else:
            lo = mid + 1
    return lo


def gen_leave(L, rng):
    out = []
    for _ in range(250):
        n_flows = int(rng.integers(1, 4))
        index = rng.choice(8, size=n_flows, replace=False).astype(np.uint64)
        flow = 10 ** rng.uniform(-7, -3, size=n_flows)
        if rng.random() < 0.1:
            flow[0] = 0.0  # a closed outlet: no draw, no exit
        vol = 10 ** rng.uniform(-4, -1, size=n_flows)
        dt = float(10 ** rng.uniform(-2, 0))
        cases = []
        for f in range(n_flows):
            kb = exit_boundary(L, dt, flow[f], vol[f]) if flow[f] > 0 else 0
            ks = [kb + d for d in (-2, -1, 0, 1)] + [int(v) for v in rng.integers(0, 1 << 23, size=2)]
            for k in ks:
                k = min(max(k, 0), (1 << 23) - 1)
                u = draw_value(k)
                status = 0 if rng.random() < 0.9 else 2
                age = float(np.float32(rng.uniform(0, 100)))
                st, ag = I32(0), F32(0)
                dead = L.ref_leave_one(n_flows, ptr(index, PU64), ptr(flow, PD), ptr(vol, PD), dt, int(index[f]),
                                       status, age, u, ct.byref(st), ct.byref(ag))
                cases.append({"pos": int(index[f]), "status": status, "age": b32(age), "u": b32(u),
                              "status_out": int(st.value), "age_out": b32(ag.value), "exits": int(dead)})
        # a particle away from every outlet
        u = draw_value(int(rng.integers(0, 1 << 23)))
        st, ag = I32(0), F32(0)
        dead = L.ref_leave_one(n_flows, ptr(index, PU64), ptr(flow, PD), ptr(vol, PD), dt, 99, 0, 1.5, u,
                               ct.byref(st), ct.byref(ag))
        cases.append({"pos": 99, "status": 0, "age": b32(1.5), "u": b32(u), "status_out": int(st.value),
                      "age_out": b32(ag.value), "exits": int(dead)})
        out.append({"index": [int(v) for v in index], "flow": [b64(v) for v in flow],
                    "volume": [b64(v) for v in vol], "dt": b64(dt), "cases": cases})
    return out


def gen_fixed_length(L, rng):
    upd, div = [], []
    for _ in range(1500):
        x = np.array([rng.uniform(0.4e-6, 2.2e-6), 2e-6 if rng.random() < 0.8 else rng.uniform(1e-6, 3e-6)],
                     dtype=np.float32)
        r = rng.random()
        s = float(rng.uniform(0, 20)) if r < 0.6 else (0.0 if r < 0.7 else float(10 ** rng.uniform(-8, -2)))
        if rng.random() < 0.05:
            s = -float(rng.uniform(0, 5e-4))  # the reference does not clamp negative concentrations
        dt = np.float32(rng.uniform(0.001, 0.5))
        x0 = x.copy()
        ctb = np.zeros(1, np.float32)
        st = L.ref_fixed_length_update(float(dt), ptr(x, PF), s, ptr(ctb, PF))
        upd.append({"dt": b32(dt), "x": [b32(v) for v in x0], "s": b64(s), "x_out": [b32(v) for v in x],
                    "ctb": b32(ctb[0]), "status": int(st)})
    for _ in range(500):
        x = np.array([rng.uniform(1e-6, 3e-6), rng.uniform(1e-6, 3e-6)], dtype=np.float32)
        x0 = x.copy()
        ch = np.zeros(2, np.float32)
        L.ref_fixed_length_division(ptr(x, PF), ptr(ch, PF))
        div.append({"x": [b32(v) for v in x0], "x_out": [b32(v) for v in x], "child": [b32(v) for v in ch]})
    return upd, div


def sa_state(rng):
    a_max = 2e-6 / 3600.0
    x = np.zeros(9, np.float32)
    x[0] = rng.uniform(0.5e-6, 2.6e-6)
    x[1] = rng.uniform(1.4e-6, 2.6e-6)
    x[2] = a_max * rng.uniform(0.05, 2.0)
    x[3] = a_max * rng.uniform(0.5, 1.5)
    x[4:] = rng.uniform(-1e-9, 1e-9, size=5)
    return x


def gen_simple_acetate(L, rng):
    upd, div, ini = [], [], []
    for _ in range(1500):
        x = sa_state(rng)
        r = rng.random()
        c0 = float(rng.uniform(0, 20)) if r < 0.5 else float(10 ** rng.uniform(-9, -1))
        c1 = float(rng.uniform(0, 2)) if rng.random() < 0.5 else float(10 ** rng.uniform(-10, -2))
        if rng.random() < 0.1:
            c0 = 0.0
        if rng.random() < 0.1:
            c1 = 0.0
        dt = np.float32(rng.uniform(0.001, 0.5))
        x0 = x.copy()
        ctb = np.zeros(2, np.float32)
        st = L.ref_simple_acetate_update(float(dt), ptr(x, PF), c0, c1, ptr(ctb, PF))
        upd.append({"dt": b32(dt), "x": [b32(v) for v in x0], "c": [b64(c0), b64(c1)],
                    "x_out": [b32(v) for v in x], "ctb": [b32(v) for v in ctb], "status": int(st)})
    for _ in range(500):
        x = sa_state(rng)
        x[4] = np.float32(rng.uniform(0.05, 1.5) * 2e-6 / 3600.0)  # a_e of the last update (> 0)
        x0 = x.copy()
        ch = np.zeros(9, np.float32)
        z = rng.normal(size=2)
        u = [draw_value(int(k)) for k in rng.integers(0, 1 << 23, size=2)]
        tape = np.array([z[0], z[1], u[0], u[1]], dtype=np.float64)
        L.ref_simple_acetate_division(ptr(x, PF), ptr(ch, PF), ptr(tape, PD), 4)
        div.append({"x": [b32(v) for v in x0], "z": [b64(v) for v in z], "u": [b32(v) for v in u],
                    "x_out": [b32(v) for v in x], "child": [b32(v) for v in ch]})
    for _ in range(300):
        x = np.zeros(9, np.float32)
        u = [draw_value(int(k)) for k in rng.integers(0, 1 << 23, size=2)]
        tape = np.array(u, dtype=np.float64)
        L.ref_simple_acetate_init(ptr(x, PF), ptr(tape, PD), 2)
        ini.append({"u": [b32(v) for v in u], "x_out": [b32(v) for v in x]})
    return upd, div, ini


def gen_distributions(L, rng):
    erf_f, erf_d, ninv, tn = [], [], [], []
    xs = np.concatenate([rng.uniform(-0.999, 0.999, 1000), [0.0, 0.5, -0.5, 0.9, -0.9, 0.99, 1e-7]])
    for x in xs:
        xf = np.float32(x)
        erf_f.append({"x": b32(xf), "y": b32(L.ref_erfinv_f(float(xf)))})
        erf_d.append({"x": b64(x), "y": b64(L.ref_erfinv_d(float(x)))})
    for _ in range(1000):
        p = np.float32(draw_value(int(rng.integers(0, 1 << 23))))
        m, s = np.float32(rng.uniform(-2, 2)), np.float32(rng.uniform(0.01, 3))
        ninv.append({"p": b32(p), "mean": b32(m), "sd": b32(s), "y": b32(L.ref_norminv_f(float(p), float(m), float(s)))})
    lm = np.float32(2e-6)
    dists = [  # the model's distributions (simple_acetate.hpp L84-L89) and random ones
        (lm, np.float32(float(lm) / 10.0), np.float32(float(lm) * 0.7), np.float32(1.3 * float(lm))),
        (np.float32(float(lm) * 0.75), np.float32(float(lm) / 10.0), np.float32(0.7 * float(np.float32(float(lm) / 2.0))),
         np.float32(float(lm) * 1.3)),
    ]
    for _ in range(1500):
        if rng.random() < 0.5:
            mu, sd, lo, hi = dists[int(rng.integers(2))]
        else:
            mu = np.float32(rng.uniform(-1, 1))
            sd = np.float32(rng.uniform(0.1, 2))
            lo = np.float32(mu - rng.uniform(0.1, 3) * sd)
            hi = np.float32(mu + rng.uniform(0.1, 3) * sd)
        u = draw_value(int(rng.integers(0, 1 << 23)))
        y = L.ref_truncnorm_f(u, float(mu), float(sd), float(lo), float(hi))
        tn.append({"u": b32(u), "mu": b32(mu), "sd": b32(sd), "lo": b32(lo), "hi": b32(hi), "y": b32(y)})
    return erf_f, erf_d, ninv, tn


def main(ref_root: str):
    L = load(ref_root)
    rng = np.random.default_rng(20261204)
    out = {"find_next": gen_find_next(L, rng), "move": gen_move(L, rng), "leave": gen_leave(L, rng)}
    out["fixed_length_update"], out["fixed_length_division"] = gen_fixed_length(L, rng)
    out["simple_acetate_update"], out["simple_acetate_division"], out["simple_acetate_init"] = \
        gen_simple_acetate(L, rng)
    out["erfinv_f"], out["erfinv_d"], out["norminv_f"], out["truncnorm_f"] = gen_distributions(L, rng)
    cd = []
    for _ in range(200):
        a = np.float32(rng.uniform(0, 3))
        b = a if rng.random() < 0.3 else np.float32(rng.uniform(0, 3))
        cd.append({"l": b32(a), "lc": b32(b), "status": int(L.ref_check_div_f(float(a), float(b)))})
    out["check_div"] = cd
    feeds = []
    for _ in range(600):
        kind = int(rng.integers(1, 3))
        f0 = float(10 ** rng.uniform(-7, -3))
        rate = float(rng.choice([-1.0, 1.0]) * 10 ** rng.uniform(-11, -7)) if kind == 1 else \
            float(rng.choice([-1.0, 1.0]) * 10 ** rng.uniform(-6, -2))
        dt = float(rng.choice([0.05, 0.1, rng.uniform(0.001, 1.0)]))
        n = int(rng.integers(0, 20000))
        t = L.ref_relative_time(dt, n)
        feeds.append({"kind": kind, "f0": b64(f0), "rate": b64(rate), "dt": b64(dt), "n": n, "t": b64(t),
                      "flow": b64(L.ref_feed_flow(kind, f0, rate, t, dt))})
    out["feed_flow"] = feeds
    out["assert_failures"] = int(L.ref_assert_failures())
    with open(os.path.join(HERE, "ref_pins.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print({k: len(v) if isinstance(v, list) else v for k, v in out.items()})


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
