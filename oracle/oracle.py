"""CPU oracle for the se_e2_a descriptor path — TEST INFRASTRUCTURE ONLY.

numpy/ctypes front end of ``liboracle.so`` (built from ``oracle/oracle.cc``,
a restatement of the reference's CPU algorithm) and, where it was built in
this checkout, of ``_ref/libref_cpu.so`` (the reference's own CPU library
compiled from its sources).  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg may import this module; the product path never
does.

Every function returns fresh numpy arrays laid out exactly as the reference's
operator contract lays them out (``source/op/tf/prod_env_mat_multi_device.cc``
outputs, ``source/lib/include/*.h`` signatures).
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS: dict[str, ctypes.CDLL] = {}

_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float


def build(ref: bool = True) -> None:
    """Compile liboracle.so (and _ref/libref_cpu.so when the reference
    sources exist) with the Makefile beside this file."""
    target = "all" if ref else "oracle"
    subprocess.run(["make", "-s", "-C", _HERE, target], check=True)


def _load(kind: str) -> ctypes.CDLL:
    if kind in _LIBS:
        return _LIBS[kind]
    path = os.path.join(_HERE, "liboracle.so" if kind == "oracle" else "_ref/libref_cpu.so")
    if not os.path.exists(path):
        if kind == "oracle":
            build(ref=False)
        else:
            raise FileNotFoundError(path)
    lib = ctypes.CDLL(path)
    _LIBS[kind] = lib
    return lib


def have_ref() -> bool:
    return os.path.exists(os.path.join(_HERE, "_ref/libref_cpu.so"))


def num_threads() -> int:
    return int(_load("oracle").or_num_threads())


def _sfx(dtype) -> str:
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def _c(a, dtype=None):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def _fn(kind: str, name: str):
    lib = _load(kind)
    pre = "or_" if kind == "oracle" else "ref_"
    return getattr(lib, pre + name)


def _sec(sel) -> np.ndarray:
    return np.concatenate([[0], np.cumsum(sel)]).astype(np.int32)


# ---------------------------------------------------------------- geometry --
def normalize_coord(coord, box, kind="oracle"):
    """source/lib/src/coord.cc:13-28 normalize_coord_cpu (one frame)."""
    c = _c(coord).copy()
    b = _c(box, c.dtype)
    _fn(kind, "normalize_coord_" + _sfx(c.dtype))(_ptr(c), _I(c.size // 3), _ptr(b))
    return c


def copy_coord(coord, atype, box, rcut, kind="oracle"):
    """source/lib/src/coord.cc:30-67 copy_coord_cpu (one frame) ->
    (ext_coord [nall,3], ext_type [nall], mapping [nall])."""
    c = _c(coord)
    t = _c(atype, np.int32)
    b = _c(box, c.dtype)
    nloc = t.size
    cap = nloc * 32 + 64
    f = _fn(kind, "copy_coord_" + _sfx(c.dtype))
    while True:
        oc = np.zeros(cap * 3, c.dtype)
        ot = np.zeros(cap, np.int32)
        om = np.zeros(cap, np.int32)
        nall = f(_ptr(oc), _ptr(ot), _ptr(om), _I(cap), _ptr(c), _ptr(t), _I(nloc),
                 _F(rcut), _ptr(b))
        if nall <= cap:
            return oc[: nall * 3].reshape(nall, 3), ot[:nall], om[:nall]
        cap = nall


def format_nlist(ext_coord, ext_type, nloc, rcut, sel, kind="oracle"):
    """build_nlist_cpu (neighbor_list.cc:873-916) + format_nlist_cpu
    (fmt_nlist.cc:145-177): [nloc, sum(sel)] int32 in the extended index space."""
    c = _c(ext_coord).reshape(-1)
    t = _c(ext_type, np.int32)
    sec = _sec(sel)
    nl = np.full(nloc * int(sec[-1]), -1, np.int32)
    _fn(kind, "format_nlist_" + _sfx(c.dtype))(
        _ptr(nl), _ptr(c), _ptr(t), _I(nloc), _I(t.size), _F(rcut), _ptr(sec),
        _I(len(sel)))
    return nl.reshape(nloc, -1)


def prod_env_mat_a_ext(ext_coord, ext_type, nloc, avg, std, rcut, rcut_smth, sel):
    """prod_env_mat_a_cpu (prod_env_mat.cc:14-108) on already-extended
    coordinates with the brute-force candidate list (oracle only)."""
    c = _c(ext_coord).reshape(-1)
    dt = c.dtype
    t = _c(ext_type, np.int32)
    sec = _sec(sel)
    nnei = int(sec[-1])
    em = np.zeros(nloc * nnei * 4, dt)
    emd = np.zeros(nloc * nnei * 12, dt)
    rij = np.zeros(nloc * nnei * 3, dt)
    nl = np.zeros(nloc * nnei, np.int32)
    a = _c(avg, dt)
    s = _c(std, dt)
    _fn("oracle", "prod_env_mat_a_" + _sfx(dt))(
        _ptr(em), _ptr(emd), _ptr(rij), _ptr(nl), _ptr(c), _ptr(t), _ptr(a), _ptr(s),
        _I(nloc), _I(t.size), _F(rcut), _F(rcut_smth), _ptr(sec), _I(len(sel)))
    return em, emd, rij, nl


def format_nlist_pt(ext_coord, ext_type, nlist_in, nloc, rcut, sel):
    """The forward_lower neighbour formatting of the PyTorch model
    (make_model.py:541-598 with extra_nlist_sort, nlist.py:304-337) on one
    frame: ext_coord [nall, 3], ext_type [nall], nlist_in [nloc, nnei_in]
    (extended indices, -1 padding).  Returns [nloc, sum(sel)] int32."""
    c = _c(ext_coord).reshape(-1)
    dt = c.dtype
    t = _c(ext_type, np.int32)
    nl = _c(nlist_in, np.int32).reshape(nloc, -1)
    sec = _sec(sel)
    out = np.zeros((nloc, int(sec[-1])), np.int32)
    _fn("oracle", "format_nlist_pt_" + _sfx(dt))(
        _ptr(out), _ptr(c), _ptr(t), _ptr(nl), _I(nloc), _I(nl.shape[1]),
        ctypes.c_double(rcut), _ptr(sec), _I(len(sel)))
    return out


def env_mat_a_nlist(ext_coord, ext_type, fmt, nloc, avg, std, rcut, rcut_smth, sel):
    """env_mat_a_cpu rows for a formatted list (prod_env_mat.cc:84-100
    normalisation): returns flat (em, em_deriv, rij)."""
    c = _c(ext_coord).reshape(-1)
    dt = c.dtype
    t = _c(ext_type, np.int32)
    f = _c(fmt, np.int32).reshape(-1)
    sec = _sec(sel)
    nnei = int(sec[-1])
    em = np.zeros(nloc * nnei * 4, dt)
    emd = np.zeros(nloc * nnei * 12, dt)
    rij = np.zeros(nloc * nnei * 3, dt)
    _fn("oracle", "env_mat_a_nlist_" + _sfx(dt))(
        _ptr(em), _ptr(emd), _ptr(rij), _ptr(c), _ptr(t), _ptr(f), _ptr(_c(avg, dt)),
        _ptr(_c(std, dt)), _I(nloc), _F(rcut), _F(rcut_smth), _ptr(sec), _I(len(sel)))
    return em, emd, rij


def prod_env_mat_a_pbc(coord, atype, box, avg, std, rcut, rcut_smth, sel,
                       map_to_local=True, kind="oracle", return_ext=False, cell_list=False):
    """The TF ProdEnvMatA op in its internal-PBC (mesh of 6) mode for ONE
    frame: normalise, copy ghosts, candidate build, format, env mat,
    normalise by davg/dstd and (optionally) map indices to local atoms.
    The candidate build is build_nlist_cpu's brute force
    (neighbor_list.cc:873-916), or with ``cell_list`` (oracle only) the O(N)
    cell list of build_nlist (neighbor_list.cc:303-420): the same candidate
    set, so the same outputs.
    Returns flat (descrpt, descrpt_deriv, rij, nlist) as the op does."""
    c = _c(coord).reshape(-1)
    dt = c.dtype
    t = _c(atype, np.int32)
    b = _c(box, dt).reshape(-1)
    nloc = t.size
    sec = _sec(sel)
    nnei = int(sec[-1])
    em = np.zeros(nloc * nnei * 4, dt)
    emd = np.zeros(nloc * nnei * 12, dt)
    rij = np.zeros(nloc * nnei * 3, dt)
    nl = np.zeros(nloc * nnei, np.int32)
    a = _c(avg, dt)
    s = _c(std, dt)
    nall = _I(0)
    cap = nloc * 32 + 64 if return_ext else 0
    ec = np.zeros(max(cap, 1) * 3, dt)
    et = np.zeros(max(cap, 1), np.int32)
    emap = np.zeros(max(cap, 1), np.int32)
    name = "prod_env_mat_a_pbc_cells_" if cell_list else "prod_env_mat_a_pbc_"
    if cell_list and kind != "oracle":
        raise ValueError("the cell-list build is an oracle restatement only")
    _fn(kind, name + _sfx(dt))(
        _ptr(em), _ptr(emd), _ptr(rij), _ptr(nl), _ptr(c), _ptr(t), _ptr(b), _ptr(a),
        _ptr(s), _I(nloc), _F(rcut), _F(rcut_smth), _ptr(sec), _I(len(sel)),
        _I(1 if map_to_local else 0), ctypes.byref(nall),
        _ptr(ec) if return_ext else None, _ptr(et), _ptr(emap), _I(cap))
    out = (em, emd, rij, nl)
    if return_ext:
        n = nall.value
        out = out + (ec[: n * 3].reshape(n, 3), et[:n], emap[:n])
    return out


# ----------------------------------------------------------------- tables --
def tabulate_fusion_se_a(table, info, em_x, em, M, kind="oracle"):
    """tabulate.cc:80-157 -> out [nloc, 4, M]."""
    tb = _c(table)
    dt = tb.dtype
    em = _c(em, dt)
    nloc, nnei = em.shape[0], em.shape[1]
    out = np.zeros(nloc * 4 * M, dt)
    _fn(kind, "tabulate_fusion_se_a_" + _sfx(dt))(
        _ptr(out), _ptr(tb), _ptr(_c(info, dt)), _ptr(_c(em_x, dt)), _ptr(em),
        _I(nloc), _I(nnei), _I(M))
    return out.reshape(nloc, 4, M)


def tabulate_fusion_se_a_grad(table, info, em_x, em, dy, kind="oracle"):
    """tabulate.cc:158-260 -> (dy_dem_x [nloc, nnei], dy_dem [nloc, nnei, 4])."""
    tb = _c(table)
    dt = tb.dtype
    em = _c(em, dt)
    dy = _c(dy, dt)
    nloc, nnei = em.shape[0], em.shape[1]
    M = dy.shape[-1]
    gx = np.zeros(nloc * nnei, dt)
    gm = np.zeros(nloc * nnei * 4, dt)
    _fn(kind, "tabulate_fusion_se_a_grad_" + _sfx(dt))(
        _ptr(gx), _ptr(gm), _ptr(tb), _ptr(_c(info, dt)), _ptr(_c(em_x, dt)), _ptr(em),
        _ptr(dy), _I(nloc), _I(nnei), _I(M))
    return gx.reshape(nloc, nnei), gm.reshape(nloc, nnei, 4)


def tabulate_fusion_se_a_grad_grad(table, info, em_x, em, dz_dem_x, dz_dem, M,
                                   kind="oracle"):
    """tabulate.cc:261-384 -> dz_dy [nloc, 4, M]."""
    tb = _c(table)
    dt = tb.dtype
    em = _c(em, dt)
    nloc, nnei = em.shape[0], em.shape[1]
    out = np.zeros(nloc * 4 * M, dt)
    _fn(kind, "tabulate_fusion_se_a_grad_grad_" + _sfx(dt))(
        _ptr(out), _ptr(tb), _ptr(_c(info, dt)), _ptr(_c(em_x, dt)), _ptr(em),
        _ptr(_c(dz_dem_x, dt)), _ptr(_c(dz_dem, dt)), _I(nloc), _I(nnei), _I(M))
    return out.reshape(nloc, 4, M)


# ------------------------------------------------------ force and virial --
def prod_force_a(net_deriv, env_deriv, nlist, nloc, nall, nnei, nframes=1,
                 kind="oracle"):
    """prod_force.cc:22-72 -> force [nframes, nall*3]."""
    g = _c(net_deriv).reshape(-1)
    dt = g.dtype
    f = np.zeros(nframes * nall * 3, dt)
    _fn(kind, "prod_force_a_" + _sfx(dt))(
        _ptr(f), _ptr(g), _ptr(_c(env_deriv, dt)), _ptr(_c(nlist, np.int32)), _I(nloc),
        _I(nall), _I(nnei), _I(nframes))
    return f.reshape(nframes, nall * 3)


def prod_virial_a(net_deriv, env_deriv, rij, nlist, nloc, nall, nnei,
                  kind="oracle"):
    """prod_virial.cc:22-68 (one frame) -> (virial [9], atom_virial [nall*9])."""
    g = _c(net_deriv).reshape(-1)
    dt = g.dtype
    v = np.zeros(9, dt)
    av = np.zeros(nall * 9, dt)
    _fn(kind, "prod_virial_a_" + _sfx(dt))(
        _ptr(v), _ptr(av), _ptr(g), _ptr(_c(env_deriv, dt)), _ptr(_c(rij, dt)),
        _ptr(_c(nlist, np.int32)), _I(nloc), _I(nall), _I(nnei))
    return v, av


def prod_force_grad_a(grad, env_deriv, nlist, nloc, nnei, nframes=1,
                      kind="oracle"):
    """prod_force_grad.cc:22-73 -> grad_net [nframes*nloc*4*nnei]."""
    gr = _c(grad).reshape(-1)
    dt = gr.dtype
    out = np.zeros(nframes * nloc * nnei * 4, dt)
    _fn(kind, "prod_force_grad_a_" + _sfx(dt))(
        _ptr(out), _ptr(gr), _ptr(_c(env_deriv, dt)), _ptr(_c(nlist, np.int32)),
        _I(nloc), _I(nnei), _I(nframes))
    return out


def prod_virial_grad_a(grad, env_deriv, rij, nlist, nloc, nnei, kind="oracle"):
    """prod_virial_grad.cc:20-66 (one frame) -> grad_net [nloc*4*nnei]."""
    gr = _c(grad).reshape(-1)
    dt = gr.dtype
    out = np.zeros(nloc * nnei * 4, dt)
    _fn(kind, "prod_virial_grad_a_" + _sfx(dt))(
        _ptr(out), _ptr(gr), _ptr(_c(env_deriv, dt)), _ptr(_c(rij, dt)),
        _ptr(_c(nlist, np.int32)), _I(nloc), _I(nnei))
    return out
