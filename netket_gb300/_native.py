"""ctypes binding of libvmck.so (the C ABI declared in include/vmck.h).

The library is built in-tree by ``netket_gb300.build``.  There is no CPU
fallback: if the library or a CUDA device is missing, every operation raises.
"""
import ctypes
import os
import threading

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libvmck.so")

F64, F32, BF16 = 0, 1, 2
DEV_NONFINITE, DEV_NOT_SPD, DEV_NO_CONVERGE, DEV_TIMEOUT, DEV_INTERNAL = 1, 2, 4, 8, 16

c_i32, c_i64, c_u64, c_dbl, c_vp = (ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64,
                                    ctypes.c_double, ctypes.c_void_p)


class VmckError(RuntimeError):
    pass


class LocalOpStruct(ctypes.Structure):
    """Mirror of ``vmck_local_op`` (include/vmck.h)."""
    _fields_ = [
        ("n_sites", c_i32), ("n_terms", c_i32), ("max_sites", c_i32), ("max_rows", c_i32),
        ("max_conns", c_i32), ("max_conn_size", c_i32), ("nonzero_diagonal", c_i32),
        ("n_groups", c_i32), ("constant", c_dbl), ("mel_cutoff", c_dbl),
        ("acting_on", c_vp), ("acting_size", c_vp), ("group_end", c_vp), ("diag_mels", c_vp),
        ("n_conns", c_vp), ("mels", c_vp), ("x_prime", c_vp),
    ]


class PauliStringsStruct(ctypes.Structure):
    """Mirror of ``vmck_pauli_strings``."""
    _fields_ = [("n_sites", c_i32), ("n_words", c_i32), ("n_flips", c_i32), ("n_strings", c_i32),
                ("cutoff", c_dbl), ("flip_mask", c_vp), ("flip_offset", c_vp),
                ("flip_site", c_vp), ("string_offset", c_vp), ("z_mask", c_vp),
                ("weight", c_vp)]


class BatchChainsStruct(ctypes.Structure):
    """Mirror of ``vmck_batch_chains``."""
    _fields_ = [("params", c_vp), ("sigma", c_vp), ("log_prob", c_vp), ("n_accepted", c_vp),
                ("samples", c_vp), ("seed", c_u64), ("counter", c_u64), ("N", c_i32),
                ("M", c_i32), ("n_chains", c_i32), ("sweep_size", c_i32)]


class BatchIsingStruct(ctypes.Structure):
    """Mirror of ``vmck_batch_ising``."""
    _fields_ = [("params", c_vp), ("x", c_vp), ("eloc", c_vp), ("edges", c_vp), ("n", c_i64),
                ("h", c_dbl), ("J", c_dbl), ("N", c_i32), ("M", c_i32), ("n_edges", c_i32),
                ("pad", c_i32)]


class OnlineStatsStruct(ctypes.Structure):
    """Mirror of ``vmck_online_stats``."""
    _fields_ = [(k, c_vp) for k in ("count", "mean", "M2", "cross", "m1", "m2", "pair", "buf")]


_SIGNATURES = {
    "vmck_abi_version": ([], c_i32),
    "vmck_error_string": ([c_i32], ctypes.c_char_p),
    "vmck_last_error": ([], ctypes.c_char_p),
    "vmck_launch_count": ([], c_i64),
    "vmck_set_wait_limit_ns": ([c_u64], c_i32),
    "vmck_wait_limit_ns": ([], c_u64),
    "vmck_ctx_create": ([ctypes.POINTER(c_vp)], c_i32),
    "vmck_ctx_destroy": ([c_vp], c_i32),
    "vmck_random_states": ([c_vp, c_vp, c_i64, c_i32, c_i32, c_u64, c_u64], c_i32),
    "vmck_get_conn_ising": ([c_vp, c_vp, c_i64, c_i32, c_vp, c_i32, c_dbl, c_dbl, c_i32, c_vp,
                             c_vp, c_vp], c_i32),
    "vmck_get_conn_local": ([c_vp, ctypes.POINTER(LocalOpStruct), c_vp, c_i64, c_vp, c_vp, c_vp],
                            c_i32),
    "vmck_get_conn_pauli": ([c_vp, ctypes.POINTER(PauliStringsStruct), c_vp, c_i64, c_vp, c_vp,
                             c_vp], c_i32),
    "vmck_rbm_eloc_pauli": ([c_vp, c_i32, c_vp, c_i32, c_i32, c_vp, c_i64,
                             ctypes.POINTER(PauliStringsStruct), c_vp, c_vp], c_i32),
    "vmck_rbm_logpsi": ([c_vp, c_i32, c_vp, c_i32, c_i32, c_vp, c_i64, c_vp, c_vp, c_vp], c_i32),
    "vmck_rbm_logpsi_tc_workspace_size": ([c_i32, c_i32, c_i64, c_i32], c_i64),
    "vmck_rbm_logpsi_tc": ([c_vp, c_vp, c_i32, c_i32, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i64,
                            c_vp], c_i32),
    "vmck_rbm_ot_v_tc_workspace_size": ([c_i32, c_i32, c_i64], c_i64),
    "vmck_rbm_ot_v_tc": ([c_vp, c_vp, c_vp, c_i32, c_i32, c_i64, c_vp, c_vp, c_vp, c_i64, c_vp],
                         c_i32),
    "vmck_eloc_from_logpsi": ([c_vp, c_i32, c_vp, c_vp, c_vp, c_i64, c_i32, c_vp], c_i32),
    "vmck_rbm_eloc_ising": ([c_vp, c_i32, c_vp, c_i32, c_i32, c_vp, c_i64, c_vp, c_i32, c_dbl,
                             c_dbl, c_vp, c_vp], c_i32),
    "vmck_rbm_eloc_local": ([c_vp, c_i32, c_vp, c_i32, c_i32, c_vp, c_i64,
                             ctypes.POINTER(LocalOpStruct), c_vp, c_vp], c_i32),
    "vmck_metropolis_sample": ([c_vp, c_i32, c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, c_i32, c_i32,
                                c_i32, c_i32, c_vp, c_u64, c_u64, c_i32, c_vp, c_i32], c_i32),
    "vmck_metropolis_hamiltonian": ([c_vp, c_i32, c_vp, c_i32, c_i32, ctypes.POINTER(LocalOpStruct),
                                     c_i32, c_vp, c_vp, c_vp, c_i32, c_i32, c_i32, c_i32, c_vp,
                                     c_u64, c_u64, c_vp], c_i32),
    "vmck_metropolis_hamiltonian_pauli": ([c_vp, c_i32, c_vp, c_i32, c_i32,
                                           ctypes.POINTER(PauliStringsStruct), c_vp, c_vp, c_vp,
                                           c_i32, c_i32, c_i32, c_i32, c_vp, c_u64, c_u64, c_vp],
                                          c_i32),
    "vmck_batched_metropolis_local": ([c_vp, c_i32, c_vp, c_i32, c_vp, c_i32, c_i32, c_vp, c_i32,
                                       c_i32, c_i32, c_i32, c_i32], c_i32),
    "vmck_batched_eloc_ising": ([c_vp, c_i32, c_vp, c_i32, c_vp, c_i32, c_i32, c_vp, c_i32, c_i32,
                                 c_i32], c_i32),
    "vmck_stats_workspace_size": ([c_i32, c_i32], c_i64),
    "vmck_stats_f64": ([c_vp, c_vp, c_i32, c_i32, c_i32, c_vp, c_vp, c_i64], c_i32),
    "vmck_stats_f64_noalloc": ([c_vp, c_vp, c_i32, c_i32, c_i32, c_vp], c_i32),
    "vmck_online_stats_update": ([c_vp, c_vp, c_i32, c_i32, c_i32, c_i32, c_dbl, c_i32,
                                  ctypes.POINTER(OnlineStatsStruct)], c_i32),
    "vmck_rbm_o_v": ([c_vp, c_i32, c_vp, c_vp, c_i32, c_i32, c_i64, c_vp, c_vp], c_i32),
    "vmck_ot_v_workspace_size": ([c_i32, c_i32, c_i64], c_i64),
    "vmck_rbm_ot_v": ([c_vp, c_i32, c_vp, c_vp, c_i32, c_i32, c_i64, c_vp, c_vp, c_vp, c_i64],
                      c_i32),
    "vmck_rbm_jacobian": ([c_vp, c_i32, c_vp, c_vp, c_i32, c_i32, c_i64, c_vp, c_dbl, c_i32,
                           c_vp], c_i32),
    "vmck_gram_workspace_size": ([c_i32, c_i32, c_i64], c_i64),
    "vmck_rbm_gram": ([c_vp, c_vp, c_i32, c_i32, c_vp, c_vp, c_i32, c_i32, c_i64, c_vp, c_dbl,
                       c_vp, c_vp, c_vp, c_i64, c_vp], c_i32),
    "vmck_gram_dense": ([c_vp, c_vp, c_i32, c_vp, c_i64, c_i64, c_i32, c_dbl, c_vp], c_i32),
    "vmck_cholesky_solve": ([c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_i64, c_vp], c_i32),
    "vmck_cholesky_solve_refined": ([c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_i32, c_dbl,
                                     c_i32, c_vp, c_vp], c_i32),
    "vmck_cholesky_solve_pcg": ([c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_i32, c_dbl, c_dbl,
                                 c_vp, c_vp, c_vp], c_i32),
    "vmck_pinv_smooth_solve": ([c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_dbl, c_dbl], c_i32),
    "vmck_center_scale": ([c_vp, c_vp, c_vp, c_i64, c_dbl, c_vp], c_i32),
    "vmck_center_update": ([c_vp, c_vp, c_vp, c_vp, c_i64, c_i64, c_dbl, c_vp], c_i32),
    "vmck_sgd": ([c_vp, c_vp, c_vp, c_i64, c_dbl, c_vp], c_i32),
    "vmck_cast_f64_f32": ([c_vp, c_vp, c_vp, c_i64], c_i32),
}

_lib = None
_lock = threading.Lock()
_ctx = {}


def lib():
    """Load libvmck.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise VmckError(f"libvmck.so is not built ({LIB_PATH}); run "
                                    "`python -m netket_gb300.build`")
                L = ctypes.CDLL(LIB_PATH)
                for name, (args, res) in _SIGNATURES.items():
                    f = getattr(L, name)
                    f.argtypes = args
                    f.restype = res
                _lib = L
    return _lib


def declared_symbols():
    return list(_SIGNATURES)


def check(rc):
    if rc != 0:
        L = lib()
        raise VmckError(f"{L.vmck_error_string(rc).decode()}: {L.vmck_last_error().decode()}")


def require_cuda():
    if not torch.cuda.is_available():
        raise VmckError("netket_gb300 needs a CUDA device (GB300, sm_103a); none is visible")


def device():
    require_cuda()
    return torch.device("cuda", torch.cuda.current_device())


def stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


_slot = threading.local()


class use_ctx:
    """Select library context ``slot`` on this thread (a context holds one
    cuBLAS / cuSOLVER handle pair and its workspace, so work that runs
    concurrently on several streams uses one slot per stream)."""

    def __init__(self, slot):
        self.slot = int(slot)

    def __enter__(self):
        self.prev = getattr(_slot, "value", 0)
        _slot.value = self.slot

    def __exit__(self, *a):
        _slot.value = self.prev


def ctx():
    """Library context of the current device and slot (cuBLAS / cuSOLVER
    handles, solver workspace)."""
    require_cuda()
    key = (torch.cuda.current_device(), getattr(_slot, "value", 0))
    if key not in _ctx:
        with _lock:
            if key not in _ctx:
                h = c_vp()
                check(lib().vmck_ctx_create(ctypes.byref(h)))
                _ctx[key] = h
    return _ctx[key]


def dtype_code(dt):
    if dt == torch.float64:
        return F64
    if dt == torch.float32:
        return F32
    raise VmckError(f"unsupported dtype {dt}")
