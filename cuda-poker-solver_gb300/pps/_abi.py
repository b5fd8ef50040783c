"""ctypes declarations of the C ABI in include/pps_gb.h (libpps_gb.so).

The library is loaded from this directory; a missing build raises
ImportError (there is no fallback implementation).
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpps_gb.so")

MAX_ACTIONS = 32
COMBOS = 1326
MAX_SIZES = 16

E_OK, E_ARG, E_INDEX, E_STATE, E_IO, E_FORMAT, E_CUDA, E_MEMORY, E_DEVICE, E_BUDGET, \
    E_TOO_WIDE, PENDING = range(12)


class BetConfig(C.Structure):
    _fields_ = [("bet_fracs", C.c_double * MAX_SIZES), ("n_bet_fracs", C.c_int),
                ("raise_mults", C.c_double * MAX_SIZES), ("n_raise_mults", C.c_int),
                ("bet_allin", C.c_int), ("bet_geometric", C.c_int), ("max_raises", C.c_int),
                ("add_allin_threshold", C.c_double), ("force_allin_threshold", C.c_double),
                ("merging_threshold", C.c_double)]


class Spot(C.Structure):
    _fields_ = [("board", C.c_uint8 * 5), ("n_board", C.c_int),
                ("oop", C.c_double * COMBOS), ("ip", C.c_double * COMBOS),
                ("pot", C.c_int64), ("stack", C.c_int64)]


class Action(C.Structure):
    _fields_ = [("kind", C.c_int32), ("amount", C.c_int64)]


class NodeStats(C.Structure):
    _fields_ = [("ev0", C.c_double), ("ev1", C.c_double), ("expl", C.c_double),
                ("pair_mass", C.c_int64)]


class Info(C.Structure):
    _fields_ = [("num_nodes", C.c_int32), ("max_depth", C.c_int32),
                ("num_decide_nodes", C.c_int32), ("iterations_run", C.c_int32),
                ("total_iterations", C.c_int64), ("n_base", C.c_int32 * 2),
                ("row_total", C.c_int64), ("empty", C.c_int32),
                ("launches_per_iteration", C.c_int32), ("device_bytes", C.c_int64),
                ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64), ("engine", C.c_int32),
                ("compensated", C.c_int32)]


class LaunchShape(C.Structure):
    _fields_ = [("plan", C.c_int32), ("fwd_cap", C.c_int32), ("bwd_cap", C.c_int32),
                ("sd_cap", C.c_int32), ("fd_cap", C.c_int32)]


class KernelStat(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_int64), ("ms", C.c_double),
                ("algo_bytes", C.c_double)]


class DecideInfo(C.Structure):
    _fields_ = [("node_id", C.c_int32), ("player", C.c_int32), ("depth", C.c_int32),
                ("n_board", C.c_int32), ("n_combos", C.c_int32), ("n_actions", C.c_int32),
                ("actions", Action * MAX_ACTIONS), ("children", C.c_int32 * MAX_ACTIONS)]


class BatchConfig(C.Structure):
    _fields_ = [("hbm_budget", C.c_int64), ("check_every", C.c_int32),
                ("fixed_checks", C.c_int32), ("max_iterations", C.c_int32),
                ("compile_threads", C.c_int32), ("algo", C.c_char * 16)]


class BatchResult(C.Structure):
    _fields_ = [("ticket", C.c_int64), ("status", C.c_int32), ("converged", C.c_int32),
                ("iterations", C.c_int32), ("num_nodes", C.c_int32), ("ev0", C.c_double),
                ("ev1", C.c_double), ("exploitability", C.c_double), ("target", C.c_double),
                ("pair_mass", C.c_int64), ("submit_ms", C.c_double), ("admit_ms", C.c_double),
                ("finish_ms", C.c_double), ("device_bytes", C.c_int64),
                ("root_actions", C.c_int32), ("root_combos", C.c_int32),
                ("root_action", Action * MAX_ACTIONS), ("root_freqs", C.c_double * MAX_ACTIONS),
                ("error", C.c_char * 160)]


class BatchInfo(C.Structure):
    _fields_ = [(k, C.c_int64) for k in (
        "submitted", "compiling", "waiting", "active", "done", "failed", "used_bytes",
        "device_bytes", "budget", "epochs", "spot_iterations", "captures", "peak_active",
        "peak_used_bytes")] + \
        [("check_every", C.c_int32), ("max_iterations", C.c_int32)] + \
        [(k, C.c_double) for k in ("admit_ms", "iterate_ms", "check_ms", "retire_ms", "idle_ms")]


ARRAY_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_char_p, C.c_char, C.c_void_p, C.c_int64)

P = C.POINTER
H = C.c_void_p
_SIGS = {
    "pps_gb_last_error": (C.c_char_p, []),
    "pps_gb_abi_version": (C.c_int, []),
    "pps_gb_bet_config_default": (None, [P(BetConfig)]),
    "pps_gb_create": (C.c_int, [P(Spot), P(BetConfig), P(H)]),
    "pps_gb_create_streets": (C.c_int, [P(Spot), P(BetConfig), P(H)]),
    "pps_gb_load": (C.c_int, [C.c_char_p, P(H)]),
    "pps_gb_destroy": (None, [H]),
    "pps_gb_solve": (C.c_int, [H, C.c_int, C.c_char_p, C.c_double]),
    "pps_gb_continue": (C.c_int, [H, C.c_int, C.c_double]),
    "pps_gb_reset": (C.c_int, [H]),
    "pps_gb_get_info": (C.c_int, [H, P(Info)]),
    "pps_gb_stats": (C.c_int, [H, P(NodeStats)]),
    "pps_gb_root_strategy": (C.c_int, [H, P(C.c_double), P(C.c_int)]),
    "pps_gb_node_strategy": (C.c_int, [H, C.c_int, P(C.c_double), P(C.c_int)]),
    "pps_gb_decide_node": (C.c_int, [H, C.c_int, P(DecideInfo)]),
    "pps_gb_combo_strategy": (C.c_int, [H, C.c_int, P(C.c_int), P(C.c_int), P(Action),
                                        P(C.c_int), P(C.c_double)]),
    "pps_gb_root_ev": (C.c_int, [H, C.c_int, P(C.c_int), P(C.c_int), P(C.c_double),
                                 P(C.c_double)]),
    "pps_gb_node_ev": (C.c_int, [H, C.c_int, P(C.c_int), P(C.c_int), P(Action), P(C.c_int),
                                 P(C.c_int), P(C.c_double), P(C.c_double), P(C.c_double),
                                 P(C.c_double), P(C.c_double)]),
    "pps_gb_runout_summary": (C.c_int, [H, C.c_int, C.c_int, P(C.c_int), P(C.c_int), P(Action),
                                        P(C.c_int), P(C.c_int), P(C.c_int), P(C.c_int),
                                        P(C.c_double), P(C.c_double)]),
    "pps_gb_player_cards": (C.c_int, [H, C.c_int, P(C.c_uint8), P(C.c_int)]),
    "pps_gb_player_weights": (C.c_int, [H, C.c_int, P(C.c_double), P(C.c_int)]),
    "pps_gb_tree_structure": (C.c_int, [H, P(C.c_uint8), P(C.c_int), P(C.c_int), P(C.c_uint8),
                                        P(C.c_int), P(C.c_int)]),
    "pps_gb_save": (C.c_int, [H, C.c_char_p]),
    "pps_gb_save_compressed": (C.c_int, [H, C.c_char_p]),
    "pps_gb_debug_dump": (C.c_int, [H]),
    "pps_gb_read_rows": (C.c_int, [H, C.c_int, P(C.c_float), C.c_int64, P(C.c_int64)]),
    "pps_gb_write_rows": (C.c_int, [H, C.c_int, P(C.c_float), C.c_int64]),
    "pps_gb_walk": (C.c_int, [H, C.c_int, C.c_int, P(C.c_double), P(C.c_double)]),
    "pps_gb_set_engine": (C.c_int, [H, C.c_int]),
    "pps_gb_set_compensated": (C.c_int, [H, C.c_int]),
    "pps_gb_set_launch_shape": (C.c_int, [H, P(LaunchShape)]),
    "pps_gb_get_launch_shape": (C.c_int, [H, P(LaunchShape)]),
    "pps_gb_time_iterations": (C.c_int, [H, C.c_int, P(C.c_double)]),
    "pps_gb_profile": (C.c_int, [H, C.c_int, C.c_int, P(KernelStat), C.c_int, P(C.c_int)]),
    "pps_gb_probe_bounded_wait": (C.c_int, [H, C.c_int]),
    "pps_gb_solve_noalloc": (C.c_int, [P(Spot), P(BetConfig), C.c_void_p, C.c_void_p, C.c_int64,
                                       C.c_int, C.c_int, C.c_void_p, P(C.c_int64)]),
    "pps_gb_batch_config_default": (None, [P(BatchConfig)]),
    "pps_gb_batch_create": (C.c_int, [P(BatchConfig), P(H)]),
    "pps_gb_batch_destroy": (None, [H]),
    "pps_gb_batch_set_budget": (C.c_int, [H, C.c_int64]),
    "pps_gb_batch_submit": (C.c_int, [H, P(Spot), P(BetConfig), C.c_int, C.c_double,
                                      P(C.c_int64)]),
    "pps_gb_batch_run": (C.c_int, [H, C.c_double]),
    "pps_gb_batch_start": (C.c_int, [H]),
    "pps_gb_batch_stop": (C.c_int, [H]),
    "pps_gb_batch_poll": (C.c_int, [H, C.c_int64, P(BatchResult)]),
    "pps_gb_batch_wait": (C.c_int, [H, C.c_int64, C.c_double, P(BatchResult)]),
    "pps_gb_batch_collect": (C.c_int, [H, P(BatchResult), C.c_int, P(C.c_int)]),
    "pps_gb_batch_root_rows": (C.c_int, [H, C.c_int64, P(C.c_float), C.c_int64,
                                         P(C.c_int64)]),
    "pps_gb_batch_get_info": (C.c_int, [H, P(BatchInfo)]),
    "pps_gb_batch_footprint": (C.c_int, [P(Spot), P(BetConfig), C.c_int, P(C.c_int64)]),
    "pps_gb_layout_digest": (C.c_int, [P(Spot), P(BetConfig), C.c_int, P(C.c_uint64)]),
    "pps_gb_compile_export": (C.c_int, [P(Spot), P(BetConfig), C.c_int, ARRAY_CB, C.c_void_p]),
    "pps_gb_hand_keys": (C.c_int, [P(C.c_uint8), C.c_int, P(C.c_uint64)]),
    "pps_gb_bet_actions": (C.c_int, [C.c_int64, C.c_int64, P(BetConfig), C.c_int64, C.c_int64,
                                     C.c_int, C.c_int, C.c_int, C.c_int, P(Action),
                                     P(C.c_int)]),
    "pps_gb_parse_range": (C.c_int, [C.c_char_p, P(C.c_double)]),
}

# Symbols include/pps_gb.h declares (the load test checks each is exported).
SYMBOLS = sorted(_SIGS)


def load_library(path: str = LIB_PATH) -> C.CDLL:
    if not os.path.exists(path):
        raise ImportError(
            "libpps_gb.so is not built (%s); run `python cuda-poker-solver_gb300/"
            "build_ext.py` (nvcc, sm_103a)" % path)
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.pps_gb_abi_version() != 1:
        raise ImportError("libpps_gb.so ABI version mismatch")
    return lib


lib = load_library()


def check(rc: int) -> None:
    if rc != E_OK:
        msg = lib.pps_gb_last_error().decode(errors="replace")
        raise RuntimeError(msg)
