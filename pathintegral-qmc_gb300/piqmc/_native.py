"""ctypes binding of ``libpiqmc_gb300.so`` (the C ABI declared in ``include/piqmc_gb300.h``).

The library is the only compute path: when it is missing, every entry point
raises ``NativeLibraryMissing``; there is no CPU fallback.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_native", "libpiqmc_gb300.so")

PQ_OK = 0
PQ_ERR_INVALID_ARG = 1
PQ_ERR_BAD_INDEX = 2
PQ_ERR_RAND_EXHAUSTED = 3
PQ_ERR_UNSUPPORTED = 4
PQ_ERR_TOO_LARGE = 5
PQ_ERR_TIMEOUT = 6
PQ_ERR_LIBC_STATE = 7
PQ_ERR_NO_DEVICE = 8

PQ_FIX_Q2 = 1
PQ_FIX_Q1 = 2
PQ_ACC_FP64 = 4


class NativeLibraryMissing(ImportError):
    pass


class PiqmcError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        msg = _strerror(status)
        super().__init__("%s%s (status %d)" % (where + ": " if where else "", msg, status))


class FastParams(ctypes.Structure):
    """Mirror of ``pq_fast_params``."""
    _fields_ = [
        ("n", ctypes.c_int), ("P", ctypes.c_int), ("R", ctypes.c_int), ("maxdeg", ctypes.c_int),
        ("nclass", ctypes.c_int), ("class_stride", ctypes.c_int), ("class_size", ctypes.c_int * 32),
        ("order_mode", ctypes.c_int), ("nsched", ctypes.c_int),
        ("mcsteps", ctypes.c_int), ("global_moves", ctypes.c_int), ("temp", ctypes.c_float),
        ("beta", ctypes.c_float), ("seed", ctypes.c_uint64), ("sweep_base", ctypes.c_int64),
        ("replica_base", ctypes.c_int), ("threads", ctypes.c_int), ("replicas_per_cta", ctypes.c_int),
    ]


class BatchRun(ctypes.Structure):
    """Mirror of ``pq_batch_run``."""
    _fields_ = [("nsched", ctypes.c_int), ("sched_base", ctypes.c_int), ("mcsteps", ctypes.c_int),
                ("global_moves", ctypes.c_int), ("order_mode", ctypes.c_int), ("beta", ctypes.c_float),
                ("sweep_base", ctypes.c_int64)]


_V, _I32, _I64, _U32, _F32, _U64 = (ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint32,
                                     ctypes.c_float, ctypes.c_uint64)

# name -> (restype, argtypes)
SIGNATURES = {
    "pq_version": (_I32, []),
    "pq_strerror": (ctypes.c_char_p, [_I32]),
    "pq_qa_sparse_reforder": (_I32, [_V, _V, _V, _I32, _I32, _I32, _I32, _I32, _V, _I32, _I32, _F32, _V, _V, _I64,
                                     _V, _I32, _V, _V]),
    "pq_qa_sparse_reforder_ex": (_I32, [_V, _V, _V, _I32, _I32, _I32, _I32, _I32, _V, _I32, _I32, _F32, _V, _V,
                                        _I64, _V, _I32, _V, _V, _I32, _V, _V, _I32, _V, _V, _V]),
    "pq_qa_dense_reforder": (_I32, [_V, _V, _I32, _I32, _I32, _V, _I32, _I32, _F32, _V, _V, _I64, _V, _I32,
                                    _V, _V]),
    "pq_qa_dense_reforder_ex": (_I32, [_V, _V, _I32, _I32, _I32, _V, _I32, _I32, _F32, _V, _V, _I64, _V,
                                       _I32, _V, _V, _I32, _V, _V, _I32, _V, _V, _V]),
    "pq_sa_sparse_reforder": (_I32, [_V, _V, _V, _I32, _I32, _I32, _V, _I32, _I32, _V, _V, _I64, _V, _V,
                                     _V]),
    "pq_sa_sparse_reforder_ex": (_I32, [_V, _V, _V, _I32, _I32, _I32, _V, _I32, _I32, _V, _V, _I64, _V, _I32,
                                        _V, _V, _I32, _V, _V, _I32, _V, _V, _V]),
    "pq_sa_dense_reforder": (_I32, [_V, _V, _I32, _I32, _V, _I32, _I32, _V, _V, _I64, _V, _V, _V]),
    "pq_sa_dense_reforder_ex": (_I32, [_V, _V, _I32, _I32, _V, _I32, _I32, _V, _V, _I64, _V, _V, _V, _I32, _V, _V,
                                       _I32, _V, _V, _V]),
    "pq_sa_bipartite_reforder_ex": (_I32, [_V, _V, _I32, _I32, _V, _V, _I32, _V, _I32, _I32, _V, _I64, _V, _V, _V,
                                           _I32, _V, _V, _I32, _V, _V, _V]),
    "pq_exp_probe": (_I32, [_V, _V, _I64, _V]),
    "pq_exp_probe_range": (_I32, [_U32, _I64, _V, _V]),
    "pq_jperp_schedule": (_I32, [_V, _I32, _I32, _F32, _V]),
    "pq_libc_rand_peek": (_I32, [_V, _I64]),
    "pq_libc_rand_skip": (_I32, [_I64]),
    "pq_host_exp": (_I32, [_V, _V, _I64]),
    "pq_host_exp_compare": (_I64, [_U32, _I64, _V, _V, _V, _I64]),
    "pq_generate_neighbors": (_I32, [_I32, _I64, _V, _V, _V, _I32, _V]),
    "pq_color_graph": (_I32, [_I32, _I32, _V, _V, _V]),
    "pq_qa_fast": (_I32, [_V, _V, _V, _V, _V, ctypes.POINTER(FastParams), _V, _V, _V]),
    "pq_qa_fast_ex": (_I32, [_V, _V, _V, _V, _V, _V, ctypes.POINTER(FastParams), _V, _V, _V]),
    "pq_batch_anneal": (_I32, [_V, _I32, _V, _V, _V, _V, _V, _V, _V, _V, _V, _V, _I32, _I32, _I32, _V, _V, _V]),
    "pq_batch_anneal_noalloc": (_I32, [_V, _I32, _V, _V, _V, _V, _V, _V, _V, _V, _V, _I32, _I32, _I32, _V, _V,
                                       _V]),
    "pq_batch_smem_bytes": (_I32, [_I32, _I32, _I32]),
    "pq_batch_occupancy": (_I32, [_I32, _I32, _V, _V]),
    "pq_tc_gemm_bf16": (_I32, [_V, _I32, _V, _I32, _V, _I32, _I32, _I32, _I32, _F32, _V, _V, _V]),
    "pq_dense_sweep": (_I32, [_V, _V, _I32, _V, _V, _I32, _V, _I32, _I32, _I32, _I32, _I32, _F32, _U64, _I64, _I32,
                              _I32, _V, _V, _V]),
    "pq_dense_sweep_ex": (_I32, [_V, _V, _I32, _V, _V, _I32, _V, _I32, _I32, _I32, _I32, _I32, _F32, _U64, _I64,
                                 _I32, _I32, _I64, _I32, _V, _V, _V]),
    "pq_dense_unpack_bf16": (_I32, [_V, _I32, _I32, _I32, _I32, _I32, _V, _V]),
    "pq_mlp_features": (_I32, [_V, _I32, _I32, _I32, _I32, _I32, _V, _V, _V, _I32, _I32, _I32, _F32, _F32, _V, _V,
                               _I64, _V]),
    "pq_mlp_relu_bf16": (_I32, [_V, _V, _I64, _V]),
    "pq_mlp_head": (_I32, [_V, _V, _F32, _V, _I64, _V]),
    "pq_mlp_propose": (_I32, [_V, _I32, _I32, _I32, _I32, _I32, _I32, _I32, _V, _V, _I64, _F32, _F32, _U32, _U64,
                              _I32, _V, _V]),
    "pq_mlp_learned_move": (_I32, [_V, _I32, _I32, _I32, _I32, _I32, _V, _V, _V, _I32, _I32, _I32, _F32, _F32, _V,
                                   _V, _V, _V, _V, _F32, _F32, _U32, _U64, _I32, _V, _V, _V, _V]),
    "pq_worldline_move": (_I32, [_V, _I32, _I32, _I32, _I32, _I32, _V, _V, _V, _I32, _I32, _I32, _F32, _U32, _U64,
                                 _I32, _V, _V]),
    "pq_mlp_learned_pass": (_I32, [_V, _I32, _I32, _I32, _I32, _I32, _V, _V, _V, _I32, _I32, _V, _F32, _F32, _V,
                                   _V, _V, _V, _V, _F32, _F32, _U32, _U64, _I32, _V, _V, _V]),
    "pq_worldline_pass": (_I32, [_V, _I32, _I32, _I32, _I32, _I32, _V, _V, _V, _I32, _I32, _V, _F32, _U32, _U64,
                                 _I32, _V, _V]),
    "pq_pair_pass": (_I32, [_V, _I32, _I32, _I32, _I32, _I32, _V, _V, _V, _V, _V, _V, _V, _I32, _F32, _U32, _U64,
                            _I32, _V, _V, _V]),
    "pq_pair_features": (_I32, [_V, _I32, _I32, _I32, _I32, _I32, _V, _V, _V, _V, _V, _V, _I32, _I32, _F32, _F32,
                                _V, _V, _I64, _V, _V]),
    "pq_pair_propose": (_I32, [_V, _I32, _I32, _I32, _I32, _V, _V, _I32, _I32, _I32, _V, _V, _I64, _F32, _F32, _U32,
                               _U64, _I32, _V, _V, _V]),
    "pq_pair_learned_pass": (_I32, [_V, _I32, _I32, _I32, _I32, _I32, _V, _V, _V, _V, _V, _V, _V, _I32, _F32, _F32,
                                    _V, _V, _V, _V, _V, _F32, _F32, _U32, _U64, _I32, _V, _V, _V]),
    "pq_generate_lattice_table": (_I32, [_I32, _I32, _I32, _I32, _I32, ctypes.c_double, ctypes.c_double, _U64,
                                         _I32, _V, _V, _V, _V]),
    "pq_mlp_head_backward": (_I32, [_V, _V, _V, _V, _I32, _V, _V, _V, _V, _V, _V]),
    "pq_mlp_hidden_backward": (_I32, [_V, _V, _I32, _V, _V, _V]),
    "pq_mlp_colsum_bf16": (_I32, [_V, _I32, _I32, _V, _V]),
    "pq_mlp_transpose_bf16": (_I32, [_V, _I32, _V, _V]),
    "pq_adam": (_I32, [_V, _V, _V, _V, _I32, _F32, _F32, _F32, _F32, _I32, _V]),
    "pq_energy_packed": (_I32, [_V, _I32, _I32, _I32, _I32, _V, _V, _V, _V, _V]),
    "pq_pack_spins": (_I32, [_V, _I32, _I32, _I32, _V, _V, _I32, _I32, _V]),
    "pq_unpack_spins": (_I32, [_V, _I32, _I32, _I32, _I32, _V, _I32, _V, _V]),
}

_lib = None


def lib():
    """Load the native library (once) and bind every signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise NativeLibraryMissing(
            "libpiqmc_gb300.so is not built (expected at %s); run "
            "`python pathintegral-qmc_gb300/build_native.py`" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _strerror(status):
    try:
        return lib().pq_strerror(int(status)).decode()
    except NativeLibraryMissing:
        return "status %d" % status


def check(status, where=""):
    if status != PQ_OK:
        raise PiqmcError(int(status), where)
