"""ctypes binding of libbmc.so (the C-ABI declared in include/bmc.h).

Loading fails loudly: there is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes as ct
import os

from . import build as _build

c_u32, c_u64, c_i32, c_dbl, c_f32 = ct.c_uint32, ct.c_uint64, ct.c_int32, ct.c_double, ct.c_float
VP = ct.c_void_p


class ModelDesc(ct.Structure):
    _fields_ = [("model", c_i32), ("f64", c_i32), ("n_var", c_u32), ("n_ctb", c_u32),
                ("params", c_dbl * 16)]


class ScenarioDesc(ct.Structure):
    _fields_ = [("model", ModelDesc), ("n_species", c_u32), ("capacity", c_u64), ("seed", c_u64),
                ("dead_ratio_threshold", c_dbl), ("min_removal", c_u64), ("value_bound", c_dbl * 8)]


class Feed(ct.Structure):
    _fields_ = [("inlet", c_u32), ("outlet", c_i32), ("flow", c_dbl), ("conc", c_dbl * 8)]


class FeedSchedule(ct.Structure):
    """bmc_feed_schedule: kind 0 constant, 1 linear f0 + t rate, 2
    exponential f0 + exp(rate t)."""
    _fields_ = [("kind", c_i32), ("pad", c_i32), ("f0", c_dbl), ("rate", c_dbl)]


class StepStats(ct.Structure):
    _fields_ = [("n_used", c_u64), ("inactive", c_u64), ("births", c_u64), ("exits", c_u64),
                ("moves", c_u64), ("overflow", c_u64), ("requested_divisions", c_u64),
                ("clamped", c_u64), ("next_id", c_u64), ("step", c_u32), ("compacted", c_u32),
                ("error", c_u32), ("pad", c_u32), ("mass_balance", c_dbl * 8)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("pad", "mass_balance")}
        d["mass_balance"] = list(self.mass_balance)
        return d


class UdfInfo(ct.Structure):
    _fields_ = [("n_var", c_u32), ("n_ctb", c_u32), ("separable", c_i32), ("has_f32", c_i32),
                ("has_f64", c_i32), ("n_names", c_u32), ("n_species", c_u32), ("pad", c_u32),
                ("names", ct.c_char_p * 16), ("species", ct.c_char_p * 8)]


RATES_FN = ct.CFUNCTYPE(None, VP, VP, VP)
UPDATE_FN = ct.CFUNCTYPE(c_i32, c_dbl, VP, VP, VP, VP)
COEF_FN = ct.CFUNCTYPE(c_dbl, VP, c_i32)
DIVISION_FN = ct.CFUNCTYPE(None, VP, VP, VP, VP)
INIT_FN = ct.CFUNCTYPE(None, VP, VP, VP)
MASS_FN = ct.CFUNCTYPE(c_dbl, VP, VP)


class UdfHostModel(ct.Structure):
    """bmc_udf_host_model: the model's functions compiled for the CPU."""
    _fields_ = [("n_var", c_u32), ("n_ctb", c_u32), ("n_rates", c_u32), ("separable", c_i32),
                ("rates", VP), ("update", VP), ("coef", VP), ("division", VP), ("init", VP),
                ("mass", VP), ("update_ctx", VP)]


class BmcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"libbmc error {code}: {msg}")
        self.code = code


_LIB = None

SIGNATURES = {
    "bmc_version": [VP, VP],
    "bmc_last_error": [],
    "bmc_device_sm_count": [VP],
    "bmc_scenario_create": [VP, VP],
    "bmc_scenario_destroy": [VP],
    "bmc_domain_update": [VP, c_u32, c_u32, VP, VP, VP, VP],
    "bmc_set_transition_coo": [VP, c_u32, c_u64, VP, VP, VP],
    "bmc_set_concentrations": [VP, VP],
    "bmc_set_feeds": [VP, c_u32, VP],
    "bmc_set_feed_schedules": [VP, c_u32, VP],
    "bmc_feed_time": [VP, VP],
    "bmc_init_particles": [VP, c_u64, c_i32, c_dbl, VP],
    "bmc_set_weight": [VP, c_dbl],
    "bmc_set_particles": [VP, c_u64, VP, VP, VP, VP, VP, VP, c_u64],
    "bmc_cycle": [VP, c_dbl, VP],
    "bmc_cycle_external": [VP, c_dbl, VP, VP, c_i32, VP],
    "bmc_step": [VP, c_dbl, VP],
    "bmc_step_enqueue": [VP, c_dbl, VP, VP],
    "bmc_step_collect": [VP],
    "bmc_run": [VP, c_dbl, c_u32, VP],
    "bmc_run_async": [VP, c_dbl, c_u32],
    "bmc_synchronize": [VP],
    "bmc_read_stats": [VP, VP],
    "bmc_read_particles": [VP, c_u64, VP, VP, VP, VP, VP, VP, VP],
    "bmc_read_liquid": [VP, VP, VP, VP],
    "bmc_repartition": [VP, VP],
    "bmc_repartition_static": [VP, VP],
    "bmc_force_remove_dead": [VP],
    "bmc_read_events": [VP, VP, c_i32],
    "bmc_read_mass": [VP, c_u64, VP, VP],
    "bmc_probe_enable": [VP, c_u64],
    "bmc_flowmap_add_gas": [VP, c_u32, VP, c_u64, VP, VP, VP, VP],
    "bmc_probe_read": [VP, c_i32, VP, c_u64, VP],
    "bmc_probe_clear": [VP, c_i32],
    "bmc_batch_create": [VP, c_u32, VP],
    "bmc_batch_create_slots": [c_u32, c_i32, c_i32, VP],
    "bmc_batch_set_slot": [VP, c_u32, VP],
    "bmc_batch_destroy": [VP],
    "bmc_batch_run": [VP, c_dbl, c_u32],
    "bmc_batch_set_shape": [VP, c_u32, c_u32, c_u32],
    "bmc_set_shape": [VP, c_u32, c_u32, c_u32],
    "bmc_set_step_limit": [VP, c_u32],
    "bmc_batch_synchronize": [VP],
    "bmc_debug_age_add": [VP, c_u64, c_dbl, VP],
    "bmc_debug_quantize": [VP, c_u64, c_i32, VP],
    "bmc_debug_draws": [c_u64, VP, c_u64, c_u32, c_u32, VP],
    "bmc_launch_count": [VP],
    "bmc_step_timed": [VP, c_dbl, VP, VP],
    "bmc_run_timed": [VP, c_dbl, c_u32, VP, VP],
    "bmc_batch_step_timed": [VP, c_dbl, VP],
    "bmc_set_device": [c_i32],
    "bmc_transfer_bytes": [VP, VP],
    "bmc_gas_set": [VP, VP, c_u64, VP, VP, VP, VP, VP],
    "bmc_gas_set_concentrations": [VP, VP],
    "bmc_gas_set_feeds": [VP, c_u32, VP],
    "bmc_gas_read": [VP, VP, VP, VP],
    "bmc_step_read": [VP, c_dbl, VP, VP],
    "bmc_reserve": [VP, c_u64],
    "bmc_debug_wait": [c_u64, c_i32, VP, VP],
    "bmc_cma_derive": [c_u32, c_u64, VP, VP, VP, VP, c_u32, VP, VP, VP],
    "bmc_cma_transition": [c_u32, c_u64, VP, VP, VP, VP, c_u64, VP, VP, VP],
    "bmc_cma_time_step": [c_dbl, c_u32, c_u32, VP, VP, VP],
    "bmc_mtr_turbulence_kla": [c_u32, VP, VP, VP, c_dbl, VP],
    "bmc_cma_read_field": [ct.c_char_p, c_u64, VP, VP],
    "bmc_cma_read_case": [ct.c_char_p, VP, VP, VP],
    "bmc_cma_case_entry": [ct.c_char_p, ct.c_uint32, VP, VP, c_u64],
    "bmc_cma_read_flowmap": [ct.c_char_p, VP, VP, VP, c_u64, VP, VP, VP],
    "bmc_flowmap_add": [VP, VP, VP, VP, VP, c_u64, VP, VP, VP],
    "bmc_flowmap_period": [VP, c_dbl],
    "bmc_flowmap_clear": [VP],
    "bmc_udf_load": [ct.c_char_p, VP],
    "bmc_udf_get_info": [c_i32, VP],
    "bmc_udf_get_host_model": [c_i32, c_i32, VP],
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libbmc.so (building it first when absent or stale)."""
    global _LIB
    if _LIB is None:
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"libbmc.so not found at {path}; run __graft_entry__.build()")
        L = ct.CDLL(path)
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ct.c_char_p if name == "bmc_last_error" else ct.c_int
        _LIB = L
    return _LIB


def check(rc: int):
    if rc != 0:
        msg = load().bmc_last_error()
        raise BmcError(rc, msg.decode() if msg else "")
    return rc


def call(name: str, *args):
    return check(getattr(load(), name)(*args))
