"""ctypes binding of libpnfft_gb300.so (the C ABI of include/pnfft.h and
include/pnfft_gb300.h).  Importing this module loads the in-tree library; it
raises if the library is missing -- there is no Python or CPU fallback."""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpnfft_gb300.so")

# flag values (include/pnfft.h)
PRE_PHI_HAT = 1 << 0
FAST_GAUSSIAN = 1 << 1
PRE_CONST_PSI = 1 << 2
PRE_LIN_PSI = 1 << 3
PRE_QUAD_PSI = 1 << 4
PRE_CUB_PSI = 1 << 5
MALLOC_F_HAT = 1 << 6
FFT_IN_PLACE = 1 << 7
INTERLACED = 1 << 8
SHIFTED_F_HAT = 1 << 9
SHIFTED_X = 1 << 10
TRANSPOSED_F_HAT = 1 << 11
DIFF_AD = 0
DIFF_IK = 1 << 12
WINDOW_KAISER_BESSEL = 0
WINDOW_GAUSSIAN = 1 << 13
WINDOW_BSPLINE = 1 << 14
WINDOW_SINC_POWER = 1 << 15
WINDOW_BESSEL_I0 = 1 << 16
USE_FK_GAUSSIAN_T = 1 << 17
WINDOW_GAUSSIAN_T = (1 << 17) | (1 << 13)
SORT_NODES = 1 << 18
FREE_F_HAT = MALLOC_F_HAT
MALLOC_NONE = 0
MALLOC_X = 1 << 0
MALLOC_F = 1 << 1
MALLOC_GRAD_F = 1 << 2
MALLOC_HESSIAN_F = 1 << 3
MALLOC_ALL = 0xF
FREE_X, FREE_F, FREE_GRAD_F, FREE_HESSIAN_F, FREE_ALL = MALLOC_X, MALLOC_F, MALLOC_GRAD_F, MALLOC_HESSIAN_F, 0xF
PRE_TENSOR = 0
PRE_FULL = 1 << 0
PRE_PSI = 1 << 1
PRE_GRAD_PSI = 1 << 2
PRE_HESSIAN_PSI = 1 << 3
COMPUTE_F = 1 << 0
COMPUTE_GRAD_F = 1 << 1
COMPUTE_HESSIAN_F = 1 << 2
COMPUTE_DIRECT = 1 << 3
COMPUTE_ACCUMULATED = 1 << 4
OMIT_DECONV = 1 << 5
OMIT_FFT = 1 << 6
OMIT_CONV = 1 << 7
TIMER_ITER, TIMER_WHOLE, TIMER_LOOP_B, TIMER_SORT_NODES, TIMER_GCELLS = 0, 1, 2, 3, 4
TIMER_MATRIX_B, TIMER_MATRIX_F, TIMER_MATRIX_D, TIMER_SHIFT_INPUT, TIMER_SHIFT_OUTPUT = 5, 6, 7, 8, 9
TIMER_LENGTH = 10
GB300_FP64 = 0
GB300_FP32_MIXED = 1
GB300_FP32 = 1 << 30
MPI_COMM_WORLD = 0x44000000
SORT_NOALLOC_MAX_NODES = 262144  # PNFFT_GB300_SORT_NOALLOC_MAX_NODES
PFFT_ESTIMATE = 1 << 0

_P = ctypes.c_void_p
_DP = ctypes.POINTER(ctypes.c_double)
_PD = ctypes.POINTER(ctypes.c_ssize_t)
_I = ctypes.c_int
_U = ctypes.c_uint
_SZ = ctypes.c_size_t
_SS = ctypes.c_ssize_t
_CS = ctypes.c_char_p
_IP = ctypes.POINTER(ctypes.c_int)
_LLP = ctypes.POINTER(ctypes.c_longlong)

# name: (restype, argtypes) for every symbol the headers declare
SIGNATURES = {
    "pnfft_create_procmesh_2d": (_I, [_I, _I, _I, _IP]),
    "pnfft_create_procmesh": (_I, [_I, _I, _IP, _IP]),
    "pnfft_local_size_3d": (None, [_PD, _I, _U, _PD, _PD, _DP, _DP]),
    "pnfft_local_size_3d_c2r": (None, [_PD, _I, _U, _PD, _PD, _DP, _DP]),
    "pnfft_local_size_adv": (None, [_I, _PD, _I, _U, _PD, _PD, _DP, _DP]),
    "pnfft_local_size_adv_c2r": (None, [_I, _PD, _I, _U, _PD, _PD, _DP, _DP]),
    "pnfft_local_size_guru": (None, [_I, _PD, _PD, _DP, _I, _I, _U, _PD, _PD, _DP, _DP]),
    "pnfft_local_size_guru_c2r": (None, [_I, _PD, _PD, _DP, _I, _I, _U, _PD, _PD, _DP, _DP]),
    "pnfft_init_3d": (_P, [_PD, _I]),
    "pnfft_init_3d_c2r": (_P, [_PD, _I]),
    "pnfft_init_adv": (_P, [_I, _PD, _U, _U, _I]),
    "pnfft_init_adv_c2r": (_P, [_I, _PD, _U, _U, _I]),
    "pnfft_init_guru": (_P, [_I, _PD, _PD, _DP, _I, _U, _U, _I]),
    "pnfft_init_guru_c2r": (_P, [_I, _PD, _PD, _DP, _I, _U, _U, _I]),
    "pnfft_init_nodes": (_P, [_SS, _U]),
    "pnfft_free_nodes": (None, [_P, _U]),
    "pnfft_precompute_psi": (None, [_P, _P, _U]),
    "pnfft_set_f": (None, [_P, _P]),
    "pnfft_set_grad_f": (None, [_P, _P]),
    "pnfft_set_hessian_f": (None, [_P, _P]),
    "pnfft_set_f_real": (None, [_P, _P]),
    "pnfft_set_grad_f_real": (None, [_P, _P]),
    "pnfft_set_hessian_f_real": (None, [_P, _P]),
    "pnfft_set_x": (None, [_P, _P]),
    "pnfft_set_f_hat": (None, [_P, _P]),
    "pnfft_set_f_hat_real": (None, [_P, _P]),
    "pnfft_set_b": (None, [ctypes.c_double, ctypes.c_double, ctypes.c_double, _P]),
    "pnfft_get_f": (_P, [_P]),
    "pnfft_get_grad_f": (_P, [_P]),
    "pnfft_get_hessian_f": (_P, [_P]),
    "pnfft_get_f_real": (_P, [_P]),
    "pnfft_get_grad_f_real": (_P, [_P]),
    "pnfft_get_hessian_f_real": (_P, [_P]),
    "pnfft_get_x": (_P, [_P]),
    "pnfft_get_f_hat": (_P, [_P]),
    "pnfft_get_f_hat_real": (_P, [_P]),
    "pnfft_get_d": (_I, [_P]),
    "pnfft_get_m": (_I, [_P]),
    "pnfft_get_x_max": (None, [_P, _DP]),
    "pnfft_get_N": (None, [_P, _PD]),
    "pnfft_get_n": (None, [_P, _PD]),
    "pnfft_get_pnfft_flags": (_U, [_P]),
    "pnfft_get_pfft_flags": (_U, [_P]),
    "pnfft_get_b": (None, [_P, _DP, _DP, _DP]),
    "pnfft_finalize": (None, [_P, _U]),
    "pnfft_trafo": (None, [_P, _P, _U]),
    "pnfft_adj": (None, [_P, _P, _U]),
    "pnfft_init": (None, []),
    "pnfft_cleanup": (None, []),
    "pnfft_malloc": (_P, [_SZ]),
    "pnfft_alloc_real": (_P, [_SZ]),
    "pnfft_alloc_complex": (_P, [_SZ]),
    "pnfft_free": (None, [_P]),
    "pnfft_init_f_hat_3d": (None, [_PD, _PD, _PD, _U, _P]),
    "pnfft_init_f": (None, [_SS, _P]),
    "pnfft_init_x_3d": (None, [_DP, _DP, _SS, _DP]),
    "pnfft_init_x_3d_adv": (None, [_DP, _DP, _DP, _SS, _DP]),
    "pnfft_zero_f_hat": (None, [_P]),
    "pnfft_inv_phi_hat": (ctypes.c_double, [_P, _I, _SS]),
    "pnfft_phi_hat": (ctypes.c_double, [_P, _I, _SS]),
    "pnfft_psi": (ctypes.c_double, [_P, _I, ctypes.c_double]),
    "pnfft_dpsi": (ctypes.c_double, [_P, _I, ctypes.c_double]),
    "pnfft_ddpsi": (ctypes.c_double, [_P, _I, ctypes.c_double]),
    "pnfft_vpr_complex": (None, [_P, _SS, _CS, _I]),
    "pnfft_vpr_real": (None, [_DP, _SS, _CS, _I]),
    "pnfft_apr_complex_3d": (None, [_P, _PD, _PD, _U, _CS, _I]),
    "pnfft_apr_real_3d": (None, [_DP, _PD, _PD, _U, _CS, _I]),
    "pnfft_get_timer_trafo": (_DP, [_P]),
    "pnfft_get_timer_adj": (_DP, [_P]),
    "pnfft_timer_average": (None, [_DP]),
    "pnfft_timer_copy": (_DP, [_DP]),
    "pnfft_timer_reduce_max": (_DP, [_I, _DP]),
    "pnfft_timer_add": (_DP, [_DP, _DP]),
    "pnfft_timer_free": (None, [_DP]),
    "pnfft_reset_timer": (None, [_P]),
    "pnfft_print_average_timer": (None, [_P, _I]),
    "pnfft_print_average_timer_adv": (None, [_P, _I]),
    "pnfft_write_average_timer": (None, [_P, _CS, _I]),
    "pnfft_write_average_timer_adv": (None, [_P, _CS, _I]),
    "pnfft_get_args": (None, [_I, _P, _CS, _I, _U, _P]),
    "pnfft_check_init_parameters": (None, [_I, _P, _PD, _PD, _PD, _IP, _P, _P, _DP, _IP, _IP, _IP]),
    "pnfft_gb300_last_error": (_CS, []),
    "pnfft_gb300_clear_error": (None, []),
    "pnfft_gb300_device_count": (_I, []),
    "pnfft_gb300_set_precision": (_I, [_P, _I]),
    "pnfft_gb300_get_precision": (_I, [_P]),
    "pnfft_gb300_set_stream": (_I, [_P, _P]),
    "pnfft_gb300_set_conv_method": (_I, [_P, _I]),
    "pnfft_gb300_get_conv_method": (_I, [_P]),
    "pnfft_gb300_get_conv_kernel": (_I, [_P, _I]),
    "pnfft_gb300_set_device_f_hat": (_I, [_P, _P]),
    "pnfft_gb300_set_device_arrays": (_I, [_P, _P, _P, _P, _P]),
    "pnfft_gb300_nodes_set_fixed": (_I, [_P, _I]),
    "pnfft_gb300_synchronize": (_I, [_P]),
    "pnfft_gb300_sort_nodes": (_I, [_P, _SS, _DP, _LLP]),
    "pnfft_gb300_node_index": (_I, [_P, _SS, _DP, _I, _LLP]),
    "pnfft_gb300_sort_nodes_noalloc": (_I, [_P, _SS, _P, _P, _P]),
    "pnfft_gb300_last_stage_ms": (_I, [_P, _I, _DP]),
    "pnfft_gb300_measure_fp32_fma": (_I, [_I, _DP]),
    "pnfft_gb300_charge_dipole": (_I, [_P, _P, _P, _U, _P, _P]),
    "pnfft_gb300_autotune": (_I, [_P, _P, _U, _U, _I]),
    "pnfft_gb300_get_tuning": (_I, [_P, ctypes.POINTER(ctypes.c_int)]),
    "pnfft_gb300_set_tuning": (_I, [_P, ctypes.POINTER(ctypes.c_int)]),
    "pnfft_gb300_batch_begin": (_I, [_P]),
    "pnfft_gb300_batch_end": (_I, []),
    "pnfft_gb300_batch_stats": (_I, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
}

_lib = None


def load():
    """Load (once) and return the ctypes handle of the in-tree library."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    return load().pnfft_gb300_last_error().decode()
