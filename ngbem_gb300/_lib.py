"""ctypes binding of libngbem_gb300.so (the C-ABI declared in include/ngbem_gb300.h).

The library must have been built (``python -c "import __graft_entry__ as g; g.build()"``);
there is no CPU fallback: importing this module without the library raises ImportError.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libngbem_gb300.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"{LIB_PATH} is missing: build the CUDA extension first "
        "(python -c 'import __graft_entry__ as g; g.build()')")

lib = C.CDLL(LIB_PATH)

BEM_OK, BEM_ERR_ARG, BEM_ERR_CUDA, BEM_ERR_ALLOC, BEM_ERR_STATE, BEM_ERR_INTERNAL = range(6)
NOALLOC_SCRATCH_BYTES = 16 << 20  # BEM_NOALLOC_SCRATCH_BYTES of include/ngbem_gb300.h
KERNELS = {"laplace_sl": 0, "laplace_dl": 1, "laplace_hs": 2, "helmholtz_sl": 3, "helmholtz_dl": 4,
           "helmholtz_hs": 5, "helmholtz_cf": 6, "maxwell_sl": 7, "helmholtz_sl_dkappa": 8,
           "maxwell_dl": 9}
KINDS = {"P0": 0, "P1": 1, "RT0": 2, "HCURL": 3, "L2P1": 4, "L2P2": 5, "L2P3": 6, "H1P2": 7, "H1P3": 8,
         "HDIV1": 9, "HDIV2": 10, "HCURL1": 11, "HCURL2": 12, "HDIV3": 13, "HDIV4": 14, "HCURL3": 15,
         "HCURL4": 16}
EVALS = {"id": 0, "rot": 1, "helm": 2, "maxwell": 3, "rotatedtrace": 4, "maxwellcurl": 5}
PRECISIONS = {"fp64": 0, "mixed": 1}
METHODS = {"aca": 0, "dense": 1}


class Params(C.Structure):
    _fields_ = [("intorder", C.c_int), ("intorder_singular", C.c_int), ("intorder_regular", C.c_int),
                ("leafsize", C.c_int), ("eta", C.c_double), ("eps", C.c_double), ("method", C.c_int),
                ("precision", C.c_int), ("max_rank", C.c_int), ("aca_eps_floor", C.c_double),
                ("scratch_bytes", C.c_longlong)]


class OperatorInfo(C.Structure):
    _fields_ = [("is_complex", C.c_int), ("height", C.c_int), ("width", C.c_int), ("nblocks", C.c_int),
                ("nnear", C.c_int), ("nfar", C.c_int), ("nfallback", C.c_int), ("nze", C.c_longlong),
                ("max_rank", C.c_int), ("sum_rank", C.c_longlong), ("bytes_dense", C.c_longlong),
                ("bytes_lowrank", C.c_longlong), ("bytes_lowrank_u", C.c_longlong), ("n_singular_pairs", C.c_int),
                ("n_regular_pairs", C.c_longlong), ("ms_setup", C.c_double), ("ms_aca", C.c_double),
                ("ms_nearfield", C.c_double), ("ms_projection", C.c_double), ("ms_total", C.c_double),
                ("mv_items", C.c_int * 4), ("mv_segments", C.c_int), ("mv_ranges", C.c_int * 4),
                ("ms_mvitems", C.c_double), ("nf_regular_evals", C.c_longlong), ("aca_evals", C.c_longlong)]


_vp, _dp, _ip, _lp = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_long)

SIGNATURES = {
    "bem_last_error": ([], C.c_char_p),
    "bem_params_default": ([C.POINTER(Params)], C.c_int),
    "bem_mesh_create": ([C.c_int, _dp, C.c_int, _ip, C.POINTER(_vp)], C.c_int),
    "bem_mesh_num_edges": ([_vp, _ip], C.c_int),
    "bem_mesh_set_geometry": ([_vp, C.c_int, _dp], C.c_int),
    "bem_mesh_destroy": ([_vp], C.c_int),
    "bem_space_create": ([_vp, C.c_int, C.c_int, C.POINTER(_vp)], C.c_int),
    "bem_space_create_on": ([_vp, C.c_int, C.c_int, _vp, C.POINTER(_vp)], C.c_int),
    "bem_space_global_dofs": ([_vp, _ip], C.c_int),
    "bem_space_element_dofs": ([_vp, _ip, _ip], C.c_int),
    "bem_space_dof_table": ([_vp, _ip, _ip], C.c_int),
    "bem_operator_autotune_tc": ([_vp, C.c_int, _ip, _dp], C.c_int),
    "bem_space_ndof": ([_vp, _ip], C.c_int),
    "bem_space_destroy": ([_vp], C.c_int),
    "bem_cluster_tree": ([_vp, C.c_int, _ip, C.c_int, _ip, _lp, _dp], C.c_int),
    "bem_partition": ([_vp, _vp, C.c_int, C.c_double, C.c_int, _ip, _ip, _ip, _ip], C.c_int),
    "bem_operator_create": ([C.c_int, C.c_double, _vp, _vp, C.c_int, C.c_int, C.POINTER(Params),
                             C.POINTER(_vp)], C.c_int),
    "bem_mass_create": ([_vp, _vp, C.c_int, C.POINTER(_vp)], C.c_int),
    "bem_operator_info": ([_vp, C.POINTER(OperatorInfo)], C.c_int),
    "bem_operator_blocks": ([_vp, _ip, _ip, _ip, _ip, _ip], C.c_int),
    "bem_operator_mult": ([_vp, C.c_int, _dp, _vp, _dp, _vp, C.c_int, _vp], C.c_int),
    "bem_operator_mult_noalloc": ([_vp, C.c_int, _dp, _vp, _dp, _vp, C.c_int, _vp], C.c_int),
    "bem_operator_mult_host": ([_vp, C.c_int, _dp, _vp, _dp, _vp, C.c_int], C.c_int),
    "bem_operator_to_dense": ([_vp, _vp], C.c_int),
    "bem_operator_status": ([_vp, _ip, C.c_int], C.c_int),
    "bem_operator_set_global_dofs": ([_vp, C.c_int, _ip, C.c_int, _ip], C.c_int),
    "bem_operator_test_waits": ([_vp, C.c_longlong, C.c_int], C.c_int),
    "bem_operator_destroy": ([_vp], C.c_int),
    "bem_operator_set_profiling": ([_vp, C.c_int], C.c_int),
    "bem_operator_set_accuracy": ([_vp, C.c_int], C.c_int),
    "bem_operator_autotune": ([_vp, C.c_int, _ip, _ip, _dp], C.c_int),
    "bem_operator_set_tensor_cores": ([_vp, C.c_int], C.c_int),
    "bem_operator_tensor_cores": ([_vp, _ip, C.POINTER(C.c_longlong), _ip, _ip, _dp], C.c_int),
    "bem_tc_selftest": ([_ip], C.c_int),
    "bem_operator_potential_dim": ([_vp, _ip], C.c_int),
    "bem_operator_set_definedon": ([_vp, _vp, _vp], C.c_int),
    "bem_operator_save": ([_vp, C.c_char_p], C.c_int),
    "bem_operator_load": ([C.c_char_p, _vp, _vp, C.POINTER(_vp)], C.c_int),
    "bem_operator_potential": ([_vp, _vp, C.c_int, _vp, _vp, _vp, _vp], C.c_int),
    "bem_operator_kernel_times": ([_vp, _dp, C.POINTER(C.c_longlong)], C.c_int),
    "bem_sl_batch_create": ([C.c_int, _ip, _ip, _ip, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(_vp)], C.c_int),
    "bem_sl_batch_eval": ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], C.c_int),
    "bem_sl_batch_info": ([_vp, _ip, _ip, C.POINTER(C.c_longlong)], C.c_int),
    "bem_sl_batch_destroy": ([_vp], C.c_int),
    "bem_gmres_batched": ([C.c_int, C.POINTER(_vp), _dp, C.c_int, _vp, _vp, C.c_int, C.c_int, C.c_double, _ip, _dp,
                           _vp], C.c_int),
    "bem_gmres": ([C.c_int, C.POINTER(_vp), _dp, _vp, _vp, C.c_int, C.c_int, C.c_double, _ip, _dp, _vp],
                  C.c_int),
}

for _name, (_args, _res) in SIGNATURES.items():
    _fn = getattr(lib, _name)
    _fn.argtypes = _args
    _fn.restype = _res


class BemError(RuntimeError):
    """Raised when a C-ABI call returns a non-zero status."""

    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def check(status: int):
    if status != BEM_OK:
        msg = lib.bem_last_error()
        raise BemError(status, msg.decode() if msg else "")
    return status


def cplx2(v) -> C.Array:
    """(re, im) pair as a ctypes double[2]."""
    z = complex(v)
    return (C.c_double * 2)(z.real, z.imag)
