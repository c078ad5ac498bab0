"""ctypes binding of ``libmoose_gb300.so`` (the C ABI in include/moose_gb300.h).

The product path is the CUDA library.  If it cannot be loaded this module
raises; there is no CPU fallback.
"""
import ctypes as C
import os

from .abi import HsBatchTuning, HsCellDesc

_LIB = None


def lib_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libmoose_gb300.so")


def load(build_if_missing=True):
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path) and build_if_missing:
        from .build import build
        build()
    if not os.path.exists(path):
        raise RuntimeError("libmoose_gb300.so is not built (run moose_gb300.build.build())")
    L = C.CDLL(path)
    vp, u32, i32, d, u64 = C.c_void_p, C.c_uint32, C.c_int, C.c_double, C.c_uint64
    pd, pu, pi = C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.POINTER(C.c_int)
    sig = {
        "hs_last_error": (C.c_char_p, []),
        "hs_device_count": (C.c_int, []),
        "hs_build_info": (C.c_char_p, []),
        "hs_create": (i32, [C.POINTER(HsCellDesc), u32, d, i32, C.POINTER(vp)]),
        "hs_destroy": (i32, [vp]),
        "hs_reinit": (i32, [vp, d]),
        "hs_process": (i32, [vp, u32]),
        "hs_process_group": (i32, [C.POINTER(vp), u32, u32]),
        "hs_set_cluster_ctas": (i32, [vp, u32]),
        "hs_get_cluster_ctas": (i32, [vp, C.POINTER(u32)]),
        "hs_sync": (i32, [vp]),
        "hs_set_ca_advance": (i32, [vp, i32]),
        "hs_get_ca_advance": (i32, [vp, pi]),
        "hs_get_table_grid": (i32, [vp, pd, pd, pi, pd, pd, pi]),
        "hs_get_nsteps": (i32, [vp, C.POINTER(u64)]),
        "hs_get_field": (i32, [vp, i32, i32, u32, pd]),
        "hs_set_field": (i32, [vp, i32, i32, u32, d]),
        "hs_set_tau_b": (i32, [vp, u32, d, d]),
        "hs_add_inject": (i32, [vp, u32, d]),
        "hs_add_gkek": (i32, [vp, u32, d, d]),
        "hs_add_conc": (i32, [vp, u32, d]),
        "hs_add_ica": (i32, [vp, u32, d]),
        "hs_push_events": (i32, [vp, pu, pd, pd, u32]),
        "hs_read_vm": (i32, [vp, pd, u32]),
        "hs_read_ca": (i32, [vp, pd, u32]),
        "hs_record": (i32, [vp, pu, u32, u32, u32]),
        "hs_read_trace": (i32, [vp, pd, u32, pu]),
        "hs_read_spikes": (i32, [vp, pu, pd, u32, pu]),
        "hs_batch_create": (i32, [C.POINTER(HsCellDesc), pu, u32, d, i32, C.POINTER(HsBatchTuning),
                                  C.POINTER(vp)]),
        "hs_batch_destroy": (i32, [vp]),
        "hs_batch_tune": (i32, [vp, C.POINTER(HsBatchTuning)]),
        "hs_batch_reinit": (i32, [vp, d]),
        "hs_batch_process": (i32, [vp, u32]),
        "hs_batch_sync": (i32, [vp]),
        "hs_batch_read_vm": (i32, [vp, u32, pd, u32]),
        "hs_batch_read_ca": (i32, [vp, u32, pd, u32]),
        "hs_batch_read_all": (i32, [vp, i32, pd, C.c_uint64]),
        "hs_read_dif": (i32, [vp, pd, u32]),
        "hs_record_values": (i32, [vp, pi, pi, pu, u32, u32, u32]),
        "hs_batch_record": (i32, [vp, pu, pu, u32, u32, u32]),
        "hs_batch_read_trace": (i32, [vp, pd, u32, pu]),
        "hs_batch_read_trace_window": (i32, [vp, u32, u32, vp]),
        "hs_batch_inject_targets": (i32, [vp, pu, pu, u32]),
        "hs_batch_set_inject": (i32, [vp, vp, u32]),
        "hs_batch_set_modulation": (i32, [vp, i32, pu, pu, pd, u32]),
        "hs_batch_read_spikes": (i32, [vp, pu, pu, pd, u32, pu]),
        "hs_batch_info": (i32, [vp, C.POINTER(u64), pu, pu, pu]),
        "hs_batch_forests": (i32, [vp, pu, pu]),
        "hs_batch_stream": (i32, [vp, C.POINTER(vp)]),
        "hs_batch_kernel_time": (i32, [vp, pd, pu]),
        "hs_batch_set_stop_steps": (i32, [vp, C.POINTER(u64), u32]),
        "hs_batch_read_steps": (i32, [vp, C.POINTER(u64), u32]),
        "hs_batch_device_bytes": (i32, [vp, C.POINTER(u64)]),
        "hs_batch_idle": (i32, [vp, pi]),
        "hs_batch_poll": (i32, [vp, u32, u32, pd, C.POINTER(u64), pu]),
        "hs_batch_set_inject_at": (i32, [vp, pu, pu, pd, u32]),
        "hs_batch_push_events": (i32, [vp, pu, pu, pd, pd, u32]),
        "hs_batch_read_spike_counts": (i32, [vp, pu, u32]),
        "hs_batch_read_cell_spikes": (i32, [vp, u32, u32, pu, pd, u32, pu]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name, None)
        if f is None:
            continue
        f.restype = res
        f.argtypes = args
    _LIB = L
    return L


class HsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("HS error %d: %s" % (code, msg))
        self.code = code


def check(rc):
    if rc != 0:
        raise HsError(rc, load().hs_last_error().decode())
    return rc


def declared_symbols(header=None):
    """Function names declared in include/moose_gb300.h."""
    import re
    if header is None:
        header = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(
            os.path.abspath(__file__)))), "include", "moose_gb300.h")
    text = open(header).read()
    return sorted(set(re.findall(r"\b(hs_[a-z0-9_]+)\s*\(", text)))
