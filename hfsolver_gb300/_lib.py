"""ctypes binding of libhfgpu.so (the C ABI of include/hfgpu.h).

The library is the only compute path: if it is missing the import fails with
an error that says how to build it; there is no CPU fallback.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhfgpu.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)

# status codes (include/hfgpu.h)
OK, ERR_INVALID, ERR_CUDA, ERR_NOT_CONVERGED, ERR_LINALG, ERR_UNSUPPORTED, ERR_NOMEM, ERR_NO_DEVICE = range(8)
MP2_NONE, MP2_FP64, MP2_SPLIT_BF16 = 0, 1, 2
SCF_MIXING, SCF_DIIS = 0, 1


class Options(ctypes.Structure):
    _fields_ = [("nscf", ctypes.c_int), ("mix_alpha", ctypes.c_double), ("tolE", ctypes.c_double),
                ("tolP", ctypes.c_double), ("scf_accel", ctypes.c_int), ("diis_size", ctypes.c_int),
                ("schwarz", ctypes.c_double), ("mp2", ctypes.c_int), ("mp2_nocc", ctypes.c_int),
                ("purify", ctypes.c_int), ("batch_streams", ctypes.c_int), ("incremental", ctypes.c_int),
                ("autotune", ctypes.c_int), ("guess", ctypes.c_int), ("eigensolver", ctypes.c_int),
                ("batch_mode", ctypes.c_int), ("reserved", ctypes.c_int * 1)]


class Result(ctypes.Structure):
    _fields_ = [("Etot", ctypes.c_double), ("E0", ctypes.c_double), ("Enuc", ctypes.c_double),
                ("Ekin", ctypes.c_double), ("E2", ctypes.c_double), ("dP", ctypes.c_double),
                ("niter", ctypes.c_int), ("nbf", ctypes.c_int), ("nocc", ctypes.c_int),
                ("nshell", ctypes.c_int), ("n_quartets", ctypes.c_int64),
                ("n_bf_quartets", ctypes.c_int64), ("n_prim_quartets", ctypes.c_int64),
                ("eri_flops", ctypes.c_double), ("ms_eri", ctypes.c_double), ("ms_scf", ctypes.c_double),
                ("ms_mp2", ctypes.c_double), ("ms_total", ctypes.c_double), ("ms_setup", ctypes.c_double),
                ("ms_fock", ctypes.c_double), ("ms_tcgemm", ctypes.c_double), ("tc_flops", ctypes.c_double),
                ("ms_grad", ctypes.c_double), ("ms_fock_full", ctypes.c_double), ("n_fock_full", ctypes.c_double),
                ("block_elems", ctypes.c_double), ("ms_tc_step1", ctypes.c_double), ("n_tc_step1", ctypes.c_double),
                ("ms_grad_eri", ctypes.c_double)]


# name -> (restype, argtypes); the list every test of the ABI checks against
_BASIS = [ctypes.c_int, _ip, _ip, _dp, _dp, _dp, _ip, _ip, _ip, ctypes.c_int, _dp, _dp]
SIGNATURES = {
    "hfgpu_last_error": (ctypes.c_char_p, []),
    "hfgpu_version": (ctypes.c_int, []),
    "hfgpu_set_stream": (ctypes.c_int, [ctypes.c_void_p]),
    "hfgpu_kernel_launches": (ctypes.c_int64, []),
    "hfgpu_probe_fp64_tflops": (ctypes.c_int, [_dp]),
    "hfgpu_getS": (ctypes.c_int, _BASIS + [_dp]),
    "hfgpu_getT": (ctypes.c_int, _BASIS + [_dp]),
    "hfgpu_getV": (ctypes.c_int, _BASIS + [ctypes.c_int, _ip, _dp, _dp, _dp, _dp]),
    "hfgpu_getInts": (ctypes.c_int, _BASIS + [_dp]),
    "hfgpu_getints2": (ctypes.c_int, [ctypes.c_int, _ip, _ip, _dp, _ip, ctypes.c_int, _dp, _dp, _dp,
                                      ctypes.c_int64]),
    "hfgpu_doscf": (ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, _dp, _dp, _dp, _dp, _ip]),
    "hfgpu_formG": (ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp]),
    "hfgpu_eigh": (ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp, _dp]),
    "hfgpu_tridiag_eigen": (ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp, _dp]),
    "hfgpu_md_flops": (ctypes.c_double, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "hfgpu_jk": (ctypes.c_int, _BASIS + [_dp, ctypes.c_double, _dp, _dp]),
    "hfgpu_mp2_energy": (ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, ctypes.c_int, _dp]),
    "hfgpu_formG_device_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p]),
    "hfgpu_transform_int2": (ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp]),
    "hfgpu_mbpt2": (ctypes.c_int, [ctypes.c_int, _dp, _dp, ctypes.c_int, _dp]),
    "hfgpu_mbpt3": (ctypes.c_int, [ctypes.c_int, _dp, _dp, ctypes.c_int, _dp]),
    "hfgpu_find_pole_diag": (ctypes.c_int, [ctypes.c_int, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, _dp, _ip]),
    "hfgpu_dgemm_sliced": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]),
    "hfgpu_default_options": (None, [ctypes.POINTER(Options)]),
    "hfgpu_basis_size": (ctypes.c_int, [ctypes.c_int, _ip]),
    "hfgpu_rhf_batch": (ctypes.c_int, [ctypes.c_int, _ip, _ip, _dp, ctypes.POINTER(Options),
                                       ctypes.POINTER(Result)]),
    "hfgpu_rhf": (ctypes.c_int, [ctypes.c_int, _ip, _dp, ctypes.POINTER(Options), ctypes.POINTER(Result), _dp,
                                 _dp]),
    "hfgpu_rhf_gradient": (ctypes.c_int, [ctypes.c_int, _ip, _dp, ctypes.POINTER(Options), ctypes.POINTER(Result),
                                          _dp]),
    "hfgpu_autotune_table": (ctypes.c_int64, [ctypes.c_char_p, ctypes.c_int64]),
    "hfgpu_autotune_clear": (None, []),
    "hfgpu_boys": (ctypes.c_int, [ctypes.c_int, ctypes.c_int64, _dp, _dp]),
    "hfgpu_grid_barrier_check": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp]),
}

_LIB = None


class HFGPUError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"hfgpu error {code}: {msg}")
        self.code = code


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built; run `python -m hfsolver_gb300.build` "
                              "(or __graft_entry__.build()) first")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def check(code):
    if code != OK:
        msg = lib().hfgpu_last_error().decode(errors="replace")
        raise HFGPUError(code, msg)
    return code
