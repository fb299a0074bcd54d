"""ctypes binding of libgbdp.so (the C ABI declared in include/gbdp.h).

The library is loaded from the package directory; there is no fallback: if
it is missing or fails to load, importing the package's operators raises.
"""

from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbdp.so")

_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_Z = ctypes.c_size_t

GBDP_OK = 0
GBDP_STATUS_CAND_OVERFLOW = 1
GBDP_STATUS = {
    1: "candidate overflow (raise max_cand)",
    2: "extended-atom overflow",
    3: "device wait timed out",
    4: "index out of range",
}


class NbrFrame(ctypes.Structure):
    _fields_ = [
        ("box", ctypes.c_double * 9),
        ("rec", ctypes.c_double * 9),
        ("boxf", ctypes.c_float * 9),
        ("recf", ctypes.c_float * 9),
        ("ncell", ctypes.c_int * 3),
        ("ngcell", ctypes.c_int * 3),
        ("stencil", ctypes.c_int * 3),
        ("nloc", ctypes.c_int),
        ("atom_off", ctypes.c_int),
        ("cell_off", ctypes.c_int),
        ("ext_cell_off", ctypes.c_int),
        ("ext_off", ctypes.c_int),
        ("ext_cap", ctypes.c_int),
        ("subcell", ctypes.c_int),
    ]


class NbrPlan(ctypes.Structure):
    _fields_ = [
        ("nframes", ctypes.c_int),
        ("nloc_total", ctypes.c_int),
        ("ncell_total", ctypes.c_int),
        ("next_cell_total", ctypes.c_int),
        ("ext_total", ctypes.c_int),
        ("max_cand", ctypes.c_int),
        ("rcut", ctypes.c_float),
        ("pad0", ctypes.c_int),
    ]


# name -> (restype, argtypes)
_SIGS = {
    "gbdp_last_error": (ctypes.c_char_p, []),
    "gbdp_version": (_I, []),
    "gbdp_selftest_wait_timeout": (_I, [_P, _P, ctypes.c_longlong, _P]),
    "gbdp_nbr_plan_make": (_I, [_P, _P, _I, _P, _P, _F, _I]),
    "gbdp_env_workspace_bytes": (_Z, [_P, _I]),
    "gbdp_env_status": (_I, [_P, _P]),
    "gbdp_prod_workspace_bytes": (_Z, [_I, _I, _I, _I, _I]),
    "gbdp_prod_env_mat_a_noalloc_f32": (_I, [_P] * 16 + [_F, _P, _I, _P]),
    "gbdp_fitting_workspace_bytes": (_Z, [_I, _P, _I, _P]),
    "gbdp_fitting_fwd_bwd_f32": (_I, [_P, _P, _P, _I, _P, _I, _P, _P, _P, _P, _F, _I, _P, _Z, _P]),
    "gbdp_prod_env_mat_a_nlist_f32": (_I, [_P] * 10 + [_I, _I, _I, _I, ctypes.c_float,
                                                        ctypes.c_float, _P, _I, _P]),
    "gbdp_prod_env_mat_a_nlist_f64": (_I, [_P] * 10 + [_I, _I, _I, _I, ctypes.c_float,
                                                        ctypes.c_float, _P, _I, _P]),
    "gbdp_frame_energy_f32": (_I, [_P, _P, _P, _I, _I, _I, _P]),
    "gbdp_frame_energy_f64": (_I, [_P, _P, _P, _I, _I, _I, _P]),
    "gbdp_table_planar_row_elems": (ctypes.c_size_t, [_I, _I]),
    "gbdp_table_to_planar_f32": (_I, [_P, _P, _I, _I, _P]),
    "gbdp_table_to_planar_f64": (_I, [_P, _P, _I, _I, _P]),
    "gbdp_se_a_descriptor_fwd_split_f32": (_I, [_P] * 9 + [_I, _P, _I, _I, _I, _I, _P]),
    "gbdp_fitting_tc_workspace_bytes": (_Z, [_I]),
    "gbdp_fitting_tc_set_persistent_min_tiles": (None, [_I]),
    "gbdp_fitting_tc_f32": (_I, [_P, _P, _P, _P, _P, _I, _P, _P, _P, _P, _Z, _P]),
    "gbdp_fitting_tc_status": (_I, [_P, _I, _P]),
    "gbdp_set_autotune": (None, [_I]),
    "gbdp_autotune_report": (_I, [ctypes.c_char_p, _I]),
    "gbdp_embed_tc_net_bytes": (_Z, []),
    "gbdp_embed_fwd_tc_bf16": (_I, [_P] * 8 + [_I, _P, _I, _P] + [_I] * 7 + [_P, _P]),
    "gbdp_embed_bwd_tc_bf16": (_I, [_P] * 8 + [_I, _P, _I, _P] + [_I] * 7 + [_P, _P]),
}


class FitTcNet(ctypes.Structure):
    _fields_ = [
        ("w_hi", _P * 3),
        ("w_lo", _P * 3),
        ("wt_hi", _P * 3),
        ("wt_lo", _P * 3),
        ("cs_fwd", _P * 3),
        ("cs_bwd", _P * 3),
        ("act_scale", ctypes.c_float * 5),
        ("b", _P * 3),
        ("idt", _P * 3),
        ("w_out", _P),
        ("b_out", ctypes.c_float),
    ]
for _s in ("f32", "f64"):
    _SIGS.update({
        f"gbdp_tabulate_fusion_se_a_{_s}": (_I, [_P, _P, _P, _P, _P, _I, _I, _I, _I, _P]),
        f"gbdp_tabulate_fusion_se_a_grad_{_s}": (_I, [_P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _P]),
        f"gbdp_tabulate_fusion_se_a_grad_grad_{_s}": (_I, [_P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _P]),
        f"gbdp_prod_env_mat_a_{_s}": (_I, [_P] * 13 + [_P, _P, _F, _P, _I, _P, _Z, _P]),
        f"gbdp_prod_env_mat_a_skin_{_s}": (_I, [_P] * 15 + [_F, _F, _P, _I, _I, _P, _P, _I, _P, _P,
                                                          _P, _Z, _P]),
        f"gbdp_prod_force_a_{_s}": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _P, _Z, _P]),
        f"gbdp_prod_virial_a_{_s}": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P, _Z, _P]),
        f"gbdp_prod_force_virial_a_{_s}": (_I, [_P] * 7 + [_I, _I, _I, _I, _I, _P, _Z, _P]),
        f"gbdp_prod_force_grad_a_{_s}": (_I, [_P, _P, _P, _P, _I, _I, _I, _P]),
        f"gbdp_prod_virial_grad_a_{_s}": (_I, [_P, _P, _P, _P, _P, _I, _I, _I, _P]),
        f"gbdp_se_a_descriptor_fwd_{_s}": (_I, [_P, _P, _P, _P, _P, _P, _P, _I, _P, _I, _I, _I, _I, _P]),
        f"gbdp_se_a_descriptor_bwd_{_s}": (_I, [_P] * 16 + [_I, _P, _I, _F, _F, _I, _I, _I, _I, _P, _P]),
    })

_lib = None


def declared_symbols() -> list[str]:
    """Every entry point declared in include/gbdp.h."""
    return sorted(_SIGS)


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with __graft_entry__.build() (nvcc, sm_103a)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class GbdpError(RuntimeError):
    pass


def check(rc: int, what: str) -> None:
    if rc != GBDP_OK:
        msg = load().gbdp_last_error().decode()
        raise GbdpError(f"{what} failed ({rc}): {msg}")


def sfx(dtype) -> str:
    import torch

    if dtype == torch.float64:
        return "f64"
    if dtype == torch.float32:
        return "f32"
    raise TypeError(f"unsupported dtype {dtype}; float32 and float64 only")


def set_autotune(on: bool) -> None:
    """Launch-shape autotuning of the fused descriptor kernels (off by
    default): the first uncaptured call per shape times each choice."""
    load().gbdp_set_autotune(1 if on else 0)


def autotune_report() -> list[str]:
    """One line per tuned shape key: kernel, dtype, sizes, the chosen warps
    per CTA (and for the backward the neighbours in flight per 16-lane group)
    and the measured milliseconds of every choice (forward: 1, 2, 4 warps;
    backward: 1, 2, 4 warps at 1 neighbour, then at 2).""" 
    lib = load()
    n = lib.gbdp_autotune_report(None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    lib.gbdp_autotune_report(buf, n + 1)
    return [l for l in buf.value.decode().splitlines() if l]
