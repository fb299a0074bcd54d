"""``torch.ops.deepmd`` operators backed by libgbdp.so (CUDA tensors only).

Schemas:
  * ``tabulate_fusion_se_a(Tensor table, Tensor table_info, Tensor em_x,
    Tensor em, int last_layer_size) -> Tensor[]`` — identical to the
    reference's op (source/op/pt/tabulate_multi_device.cc:1498-1504,
    :1550-1552): dtype from ``table``, ``table_info`` read on the host,
    autograd to em_x/em, and grad-of-grad to dy (the reference's
    TabulateFusionSeAGradOp::backward, :660-700).
  * ``prod_env_mat_a``, ``prod_force_se_a``, ``prod_virial_se_a`` — new
    PyTorch schemas mirroring the TF ops ProdEnvMatA
    (source/op/tf/prod_env_mat_multi_device.cc:11-28), ProdForceSeA
    (source/op/tf/prod_force_multi_device.cc:6-14) and ProdVirialSeA
    (source/op/tf/prod_virial_multi_device.cc:5-15).
  * ``prod_env_mat_a_nlist`` — the same outputs from an external neighbour
    list (the forward_lower path: extended coordinates and an unsorted
    rcut + skin list from an MD engine), formatted as the PyTorch model does.
  * ``enable_mpi() -> Tensor`` — present because deepmd/pt/cxx_op.py probes
    it (source/op/pt/print_summary.cc:14); always false here.

There is no CPU implementation: CPU tensors raise.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib as L

_P = ctypes.c_void_p


def _ptr(t: torch.Tensor | None):
    """Device address for a library call.  The tensor must stay referenced
    until the call has been enqueued: pass locals, never temporaries such as
    ``x.to(dtype)``, whose memory the caching allocator may hand to the next
    temporary before the kernel runs."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _need_cuda(*ts):
    for t in ts:
        if t is not None and not t.is_cuda:
            raise RuntimeError(
                "the GB300 deepmd operators run on CUDA tensors only (got a CPU tensor); "
                "there is no CPU fallback")


def _host_info(table_info: torch.Tensor, dtype, table: torch.Tensor | None = None) -> ctypes.Array:
    vals = table_info.detach().to("cpu", torch.float64).reshape(-1).tolist()
    if len(vals) < 5:
        raise RuntimeError("table_info must hold at least 5 values")
    if not (vals[3] > 0 and vals[4] > 0):
        raise RuntimeError("table strides must be positive")
    npd = np.float64 if dtype == torch.float64 else np.float32
    lo, up, mx, s0, s1 = (npd(v) for v in vals[:5])
    # the last row any x can map to, formed in the table's precision as the
    # kernels form it; a smaller table would be read out of bounds
    last = int(npd(up - lo) / s0) + int(npd(mx - up) / s1) - 1
    if table is not None and table.shape[0] <= last:
        raise RuntimeError(f"table has {table.shape[0]} rows but table_info addresses row {last}")
    ct = ctypes.c_double if dtype == torch.float64 else ctypes.c_float
    return (ct * len(vals))(*vals)


# ------------------------------------------------------------- tabulate --
def tabulate_forward(table, table_info, em_x, em, last_layer_size):
    _need_cuda(table, em_x, em)
    if table.dim() != 2:
        raise RuntimeError("Dim of table should be 2")
    if em_x.dim() != 2:
        raise RuntimeError("Dim of input should be 2")
    if em.dim() != 3:
        raise RuntimeError("Dim of input should be 3")
    dt = table.dtype
    table = table.contiguous()
    em_x = em_x.to(dt).contiguous()
    em = em.to(dt).contiguous()
    nloc, nnei = em.shape[0], em.shape[1]
    out = torch.empty((nloc, 4, last_layer_size), dtype=dt, device=table.device)
    info = _host_info(table_info, dt, table)
    fn = getattr(L.load(), f"gbdp_tabulate_fusion_se_a_{L.sfx(dt)}")
    L.check(fn(_ptr(out), _ptr(table), info, _ptr(em_x), _ptr(em), nloc, nnei,
               int(last_layer_size), 1, _stream()), "tabulate_fusion_se_a")
    return out


def tabulate_grad(table, table_info, em_x, em, dy):
    _need_cuda(table, em_x, em, dy)
    if dy.dim() != 3:
        raise RuntimeError("Dim of dy_tensor should be 3")
    dt = table.dtype
    em_x = em_x.to(dt).contiguous()
    em = em.to(dt).contiguous()
    dy = dy.to(dt).contiguous()
    nloc, nnei = em.shape[0], em.shape[1]
    gx = torch.empty_like(em_x)
    gm = torch.empty_like(em)
    info = _host_info(table_info, dt, table)
    table = table.contiguous()
    fn = getattr(L.load(), f"gbdp_tabulate_fusion_se_a_grad_{L.sfx(dt)}")
    L.check(fn(_ptr(gx), _ptr(gm), _ptr(table), info, _ptr(em_x), _ptr(em), _ptr(dy),
               nloc, nnei, dy.shape[2], 1, _stream()), "tabulate_fusion_se_a_grad")
    return gx, gm


def tabulate_grad_grad(table, table_info, em_x, em, dz_dem_x, dz_dem, last_layer_size):
    _need_cuda(table, em_x, em, dz_dem_x, dz_dem)
    dt = table.dtype
    em_x = em_x.to(dt).contiguous()
    em = em.to(dt).contiguous()
    nloc, nnei = em.shape[0], em.shape[1]
    dz = torch.empty((nloc, 4, last_layer_size), dtype=dt, device=table.device)
    info = _host_info(table_info, dt, table)
    table = table.contiguous()
    dz_dem_x = dz_dem_x.to(dt).contiguous()
    dz_dem = dz_dem.to(dt).contiguous()
    fn = getattr(L.load(), f"gbdp_tabulate_fusion_se_a_grad_grad_{L.sfx(dt)}")
    L.check(fn(_ptr(dz), _ptr(table), info, _ptr(em_x), _ptr(em), _ptr(dz_dem_x), _ptr(dz_dem),
               nloc, nnei, int(last_layer_size), 1, _stream()), "tabulate_fusion_se_a_grad_grad")
    return dz


class _TabulateGradFn(torch.autograd.Function):
    """dy -> (dy_dem_x, dy_dem); its backward is the grad-grad kernel, which
    (as in the reference) differentiates wrt dy only."""

    @staticmethod
    def forward(ctx, table, table_info, em_x, em, dy):
        ctx.save_for_backward(table, table_info, em_x, em)
        ctx.M = dy.shape[2]
        return tabulate_grad(table, table_info, em_x, em, dy)

    @staticmethod
    def backward(ctx, g_dem_x, g_dem):
        table, table_info, em_x, em = ctx.saved_tensors
        if g_dem_x is None:
            g_dem_x = torch.zeros_like(em_x)
        if g_dem is None:
            g_dem = torch.zeros_like(em)
        dz = tabulate_grad_grad(table, table_info, em_x, em, g_dem_x, g_dem, ctx.M)
        return None, None, None, None, dz


class TabulateFusionSeAFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, table, table_info, em_x, em, last_layer_size):
        ctx.save_for_backward(table, table_info, em_x, em)
        return tabulate_forward(table, table_info, em_x, em, last_layer_size)

    @staticmethod
    def backward(ctx, dy):
        table, table_info, em_x, em = ctx.saved_tensors
        gx, gm = _TabulateGradFn.apply(table, table_info, em_x, em, dy.contiguous())
        return None, None, gx, gm, None


def tabulate_fusion_se_a(table, table_info, em_x, em, last_layer_size: int):
    return [TabulateFusionSeAFn.apply(table, table_info, em_x, em, int(last_layer_size))]


# ------------------------------------------------------- neighbour plan --
class NeighborPlan:
    """Host plan + device frame table + workspace for the periodic env-mat
    pipeline of a packed batch of frames (possibly ragged)."""

    def __init__(self, nloc_per_frame, boxes, rcut: float, device, dtype=torch.float32,
                 max_cand: int = 0):
        nl = np.ascontiguousarray(np.asarray(nloc_per_frame, dtype=np.int32).reshape(-1))
        bx = np.asarray(boxes, dtype=np.float64).reshape(len(nl), 9)
        if dtype == torch.float32:
            # float coordinates come with a float box: the reference builds
            # its cell grid and ghost shifts from that box converted to
            # double (source/lib/src/coord.cc:42-47)
            bx = bx.astype(np.float32).astype(np.float64)
        bx = np.ascontiguousarray(bx)
        self.nframes = len(nl)
        self.nloc = nl
        self.boxes = bx
        self.rcut = float(rcut)
        self.dtype = dtype
        self.device = torch.device(device)
        self.plan = L.NbrPlan()
        frames = (L.NbrFrame * self.nframes)()
        lib = L.load()
        L.check(lib.gbdp_nbr_plan_make(ctypes.byref(self.plan), frames, self.nframes,
                                       nl.ctypes.data_as(_P), bx.ctypes.data_as(_P),
                                       ctypes.c_float(self.rcut), int(max_cand)),
                "nbr_plan_make")
        self.frames_host = frames
        raw = np.frombuffer(bytes(frames), dtype=np.uint8)
        self.frames_dev = torch.from_numpy(raw.copy()).to(self.device)
        fp64 = 1 if dtype == torch.float64 else 0
        self.ws_bytes = int(lib.gbdp_env_workspace_bytes(ctypes.byref(self.plan), fp64))
        self.workspace = torch.empty(self.ws_bytes, dtype=torch.uint8, device=self.device)
        p = self.plan
        self.ext_total = p.ext_total
        self.nloc_total = p.nloc_total
        self.atom_off = np.array([frames[f].atom_off for f in range(self.nframes)], np.int64)
        self.ext_off = np.array([frames[f].ext_off for f in range(self.nframes)], np.int64)

    def frame(self, f: int):
        return self.frames_host[f]

    # the candidate buffer lives in shared memory: 4 warps x max_cand x 9 B
    # per CTA, at most 4096 candidates a centre (within 200 KiB)
    MAX_CAND_LIMIT = 4096

    @property
    def max_cand(self) -> int:
        return int(self.plan.max_cand)

    def grow_candidates(self) -> bool:
        """Double the per-centre candidate capacity after a candidate
        overflow (as the reference doubles its neighbour capacity and
        retries, source/op/tf/prod_env_mat_multi_device.cc:1583-1605).  The
        workspace does not depend on it; a graph captured with the old
        capacity must be captured again.  False when the limit is reached."""
        if self.plan.max_cand >= self.MAX_CAND_LIMIT:
            return False
        self.plan.max_cand = min(2 * self.plan.max_cand, self.MAX_CAND_LIMIT)
        return True


class EnvMatResult:
    __slots__ = ("em", "em_deriv", "rij", "nlist", "nlist_ext", "ext_coord", "ext_type",
                 "ext_map", "ext_nall")


def env_mat_packed(plan: NeighborPlan, coord, atype, avg, std, rcut_smth, sel,
                   need_deriv=True, need_rij=True, need_nlist_ext=False, check_status=True,
                   out: EnvMatResult | None = None) -> EnvMatResult:
    """Run the periodic neighbour build + env matrix on a packed batch.
    coord [nloc_total, 3], atype [nloc_total] int32, avg/std [ntypes, nnei*4].
    With ``out`` given, its buffers are reused (no allocation)."""
    _need_cuda(coord, atype, avg, std)
    dt = plan.dtype
    dev = plan.device
    nnei = int(sum(sel))
    n = plan.nloc_total
    r = out
    if r is None:
        r = EnvMatResult()
        r.em = torch.empty((n, nnei, 4), dtype=dt, device=dev)
        r.em_deriv = torch.empty((n, nnei, 4, 3), dtype=dt, device=dev) if need_deriv else None
        r.rij = torch.empty((n, nnei, 3), dtype=dt, device=dev) if need_rij else None
        r.nlist = torch.empty((n, nnei), dtype=torch.int32, device=dev)
        r.nlist_ext = torch.empty((n, nnei), dtype=torch.int32, device=dev) if need_nlist_ext else None
        r.ext_coord = torch.empty((plan.ext_total, 3), dtype=dt, device=dev)
        r.ext_type = torch.empty((plan.ext_total,), dtype=torch.int32, device=dev)
        r.ext_map = torch.empty((plan.ext_total,), dtype=torch.int32, device=dev)
        r.ext_nall = torch.empty((plan.nframes,), dtype=torch.int32, device=dev)
    selc = (ctypes.c_int * len(sel))(*[int(s) for s in sel])
    fn = getattr(L.load(), f"gbdp_prod_env_mat_a_{L.sfx(dt)}")
    while True:
        L.check(fn(_ptr(r.em), _ptr(r.em_deriv), _ptr(r.rij), _ptr(r.nlist), _ptr(r.nlist_ext),
                   _ptr(r.ext_coord), _ptr(r.ext_type), _ptr(r.ext_map), _ptr(r.ext_nall),
                   _ptr(coord), _ptr(atype), _ptr(avg), _ptr(std), ctypes.byref(plan.plan),
                   _ptr(plan.frames_dev), ctypes.c_float(rcut_smth), selc, len(sel),
                   _ptr(plan.workspace), ctypes.c_size_t(plan.ws_bytes), _stream()),
                "prod_env_mat_a")
        if not check_status:
            return r
        st = L.load().gbdp_env_status(_ptr(plan.workspace), _stream())
        # a centre with more candidates than the capacity: double it and run
        # again (the outputs of the failed run are overwritten)
        if st == L.GBDP_STATUS_CAND_OVERFLOW and plan.grow_candidates():
            continue
        if st != 0:
            raise L.GbdpError(f"prod_env_mat_a device status {st}: {L.GBDP_STATUS.get(st, '?')}"
                              + (f" at max_cand {plan.max_cand}"
                                 if st == L.GBDP_STATUS_CAND_OVERFLOW else ""))
        return r


class VerletList:
    """Buffers of the skin form of the env pipeline (kept between calls):
    per centre up to ``cap`` extended indices within rcut + skin of the last
    rebuild, their count, and each extended slot's source atom and shift."""

    def __init__(self, plan: NeighborPlan, cap: int = 0):
        dev, dt = plan.device, plan.dtype
        self.cap = int(cap) if cap > 0 else plan.max_cand
        n, ne = plan.nloc_total, plan.ext_total
        self.idx = torch.empty((n, self.cap), dtype=torch.int32, device=dev)
        self.cnt = torch.zeros((n,), dtype=torch.int32, device=dev)
        self.shift = torch.empty((ne, 3), dtype=dt, device=dev)
        self.src = torch.full((ne,), -1, dtype=torch.int32, device=dev)


def env_mat_skin(plan: NeighborPlan, vl: VerletList, coord, atype, avg, std, rcut: float,
                 rcut_smth, sel, rebuild: bool, out: EnvMatResult,
                 check_status: bool = False) -> EnvMatResult:
    """The env pipeline on a Verlet list: ``plan`` made with rcut + skin;
    ``rebuild`` rebuilds ghosts and the list, otherwise the ghosts follow
    the local atoms and the list of the last rebuild is formatted at rcut.
    Outputs go to ``out`` (no allocation)."""
    _need_cuda(coord, atype, avg, std)
    dt = plan.dtype
    selc = (ctypes.c_int * len(sel))(*[int(s) for s in sel])
    fn = getattr(L.load(), f"gbdp_prod_env_mat_a_skin_{L.sfx(dt)}")
    r = out
    L.check(fn(_ptr(r.em), _ptr(r.em_deriv), _ptr(r.rij), _ptr(r.nlist), _ptr(r.nlist_ext),
               _ptr(r.ext_coord), _ptr(r.ext_type), _ptr(r.ext_map), _ptr(r.ext_nall),
               _ptr(coord), _ptr(atype), _ptr(avg), _ptr(std), ctypes.byref(plan.plan),
               _ptr(plan.frames_dev), ctypes.c_float(rcut), ctypes.c_float(rcut_smth), selc,
               len(sel), int(bool(rebuild)), _ptr(vl.idx), _ptr(vl.cnt), vl.cap, _ptr(vl.shift),
               _ptr(vl.src), _ptr(plan.workspace), ctypes.c_size_t(plan.ws_bytes), _stream()),
            "prod_env_mat_a_skin")
    if check_status:
        st = L.load().gbdp_env_status(_ptr(plan.workspace), _stream())
        if st != 0:
            raise L.GbdpError(f"prod_env_mat_a_skin device status {st}: "
                              f"{L.GBDP_STATUS.get(st, '?')}")
    return r


# ---------------------------------------------------- TF-contract ops --
_PLAN_CACHE: dict = {}


def _plan_for(nloc, boxes_np, rcut, device, dtype):
    key = (int(nloc), boxes_np.tobytes(), float(rcut), str(device), dtype)
    p = _PLAN_CACHE.get(key)
    if p is None:
        if len(_PLAN_CACHE) > 16:
            _PLAN_CACHE.clear()
        p = NeighborPlan([nloc] * boxes_np.shape[0], boxes_np, rcut, device, dtype)
        _PLAN_CACHE[key] = p
    return p


def prod_env_mat_a_impl(coord, atype, natoms, box, mesh, davg, dstd, rcut_a: float,
                        rcut_r: float, rcut_r_smth: float, sel_a, sel_r):
    """TF ProdEnvMatA in its internal-PBC mode (mesh of 6 ints).  The box is
    read on the host to plan the cell grid, as the reference does."""
    _need_cuda(coord, atype, davg, dstd)
    if any(int(s) != 0 for s in sel_r):
        raise RuntimeError("Rotational free descriptor only support all-angular information: "
                           "sel_r should be all zero.")
    nat = [int(v) for v in natoms.reshape(-1).tolist()]
    nloc, nall = nat[0], nat[1]
    ntypes = len(nat) - 2
    if mesh.numel() != 6:
        raise NotImplementedError(
            "only the internal periodic mode (mesh of 6) is implemented on GB300")
    if nloc != nall:
        raise RuntimeError("internal periodic mode requires nloc == nall")
    if len(sel_a) != ntypes:
        raise RuntimeError("number of types should match the length of sel array")
    nf = coord.shape[0]
    dt = coord.dtype
    boxes = box.detach().to("cpu", torch.float64).reshape(nf, 9).numpy()
    plan = _plan_for(nloc, boxes, rcut_r, coord.device, dt)
    nnei = int(sum(sel_a))
    r = env_mat_packed(plan, coord.reshape(nf * nloc, 3).contiguous(),
                       atype.reshape(nf * nloc).to(torch.int32).contiguous(),
                       davg.to(dt).contiguous(), dstd.to(dt).contiguous(), rcut_r_smth,
                       [int(s) for s in sel_a])
    return [r.em.reshape(nf, nloc * nnei * 4), r.em_deriv.reshape(nf, nloc * nnei * 12),
            r.rij.reshape(nf, nloc * nnei * 3), r.nlist.reshape(nf, nloc * nnei)]


def prod_env_mat_a_nlist_impl(coord, atype, nlist, davg, dstd, rcut: float, rcut_smth: float,
                              sel):
    """prod_env_mat_a from an external neighbour list (the forward_lower
    path): coord [nf, nall * 3] or [nf, nall, 3] extended coordinates with the
    nloc local atoms first, type [nf, nall], nlist [nf, nloc, nnei_in]
    extended indices (-1 padding, unsorted, rcut + skin allowed).  Formats
    the list as deepmd/pt/model/model/make_model.py:541-598 with the forced
    sort, then deepmd/pt/utils/nlist.py:304-337, and returns the ProdEnvMatA
    outputs (descrpt, descrpt_deriv, rij, nlist) with nlist in the extended
    index space."""
    _need_cuda(coord, atype, nlist, davg, dstd)
    nf, nloc, nnei_in = (int(x) for x in nlist.shape)
    dt = coord.dtype
    nall = coord.reshape(nf, -1).shape[1] // 3
    if atype.reshape(nf, -1).shape[1] != nall:
        raise RuntimeError("type must have nall entries per frame")
    sel = [int(x) for x in sel]
    nnei = sum(sel)
    dev = coord.device
    em = torch.empty((nf, nloc * nnei * 4), dtype=dt, device=dev)
    emd = torch.empty((nf, nloc * nnei * 12), dtype=dt, device=dev)
    rij = torch.empty((nf, nloc * nnei * 3), dtype=dt, device=dev)
    nl_out = torch.empty((nf, nloc * nnei), dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    sel_c = (ctypes.c_int * len(sel))(*sel)
    # converted copies stay referenced until the launch is enqueued
    coord = coord.contiguous()
    atype = atype.to(torch.int32).contiguous()
    nlist = nlist.to(torch.int32).contiguous()
    davg = davg.to(dt).contiguous()
    dstd = dstd.to(dt).contiguous()
    fn = getattr(L.load(), f"gbdp_prod_env_mat_a_nlist_{L.sfx(dt)}")
    L.check(fn(_ptr(em), _ptr(emd), _ptr(rij), _ptr(nl_out), _ptr(status), _ptr(coord),
               _ptr(atype), _ptr(nlist), _ptr(davg), _ptr(dstd), nf, nloc, nall, nnei_in,
               ctypes.c_float(rcut), ctypes.c_float(rcut_smth), sel_c, len(sel), _stream()),
            "prod_env_mat_a_nlist")
    st = int(status.item())
    if st:
        raise L.GbdpError(f"prod_env_mat_a_nlist device status {st}: "
                          f"{L.GBDP_STATUS.get(st, '?')}")
    return [em, emd, rij, nl_out]


def prod_force_se_a_impl(net_deriv, in_deriv, nlist, natoms, n_a_sel: int, n_r_sel: int,
                         deterministic: bool = False):
    _need_cuda(net_deriv, in_deriv, nlist)
    nat = [int(v) for v in natoms.reshape(-1).tolist()]
    nloc, nall = nat[0], nat[1]
    nf = net_deriv.shape[0]
    nnei = int(n_a_sel) + int(n_r_sel)
    dt = net_deriv.dtype
    force = torch.empty((nf, nall * 3), dtype=dt, device=net_deriv.device)
    lib = L.load()
    wsb = int(lib.gbdp_prod_workspace_bytes(nf, nloc, nall, nnei, int(deterministic)))
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=net_deriv.device)
    fn = getattr(lib, f"gbdp_prod_force_a_{L.sfx(dt)}")
    net_deriv = net_deriv.contiguous()
    in_deriv = in_deriv.to(dt).contiguous()
    nlist = nlist.to(torch.int32).contiguous()
    L.check(fn(_ptr(force), _ptr(net_deriv), _ptr(in_deriv), _ptr(nlist), nloc, nall, nnei, nf,
               int(deterministic), _ptr(ws), ctypes.c_size_t(wsb), _stream()), "prod_force_se_a")
    return force


def prod_virial_se_a_impl(net_deriv, in_deriv, rij, nlist, natoms, n_a_sel: int, n_r_sel: int,
                          deterministic: bool = False):
    _need_cuda(net_deriv, in_deriv, rij, nlist)
    nat = [int(v) for v in natoms.reshape(-1).tolist()]
    nloc, nall = nat[0], nat[1]
    nf = net_deriv.shape[0]
    nnei = int(n_a_sel) + int(n_r_sel)
    dt = net_deriv.dtype
    virial = torch.empty((nf, 9), dtype=dt, device=net_deriv.device)
    atom_virial = torch.empty((nf, nall * 9), dtype=dt, device=net_deriv.device)
    lib = L.load()
    wsb = int(lib.gbdp_prod_workspace_bytes(nf, nloc, nall, nnei, int(deterministic)))
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=net_deriv.device)
    fn = getattr(lib, f"gbdp_prod_virial_a_{L.sfx(dt)}")
    net_deriv = net_deriv.contiguous()
    in_deriv = in_deriv.to(dt).contiguous()
    rij = rij.to(dt).contiguous()
    nlist = nlist.to(torch.int32).contiguous()
    L.check(fn(_ptr(virial), _ptr(atom_virial), _ptr(net_deriv), _ptr(in_deriv), _ptr(rij),
               _ptr(nlist), nloc, nall, nnei, nf, int(deterministic), _ptr(ws),
               ctypes.c_size_t(wsb), _stream()), "prod_virial_se_a")
    return virial, atom_virial


def prod_force_virial_se_a_impl(net_deriv, in_deriv, rij, nlist, natoms, n_a_sel: int,
                                n_r_sel: int, deterministic: bool = False):
    """prod_force_se_a and prod_virial_se_a in one pass over their shared
    inputs: (force [nf, nall*3], virial [nf, 9], atom_virial [nf, nall*9])."""
    _need_cuda(net_deriv, in_deriv, rij, nlist)
    nat = [int(v) for v in natoms.reshape(-1).tolist()]
    nloc, nall = nat[0], nat[1]
    nf = net_deriv.shape[0]
    nnei = int(n_a_sel) + int(n_r_sel)
    dt = net_deriv.dtype
    dev = net_deriv.device
    force = torch.empty((nf, nall * 3), dtype=dt, device=dev)
    virial = torch.empty((nf, 9), dtype=dt, device=dev)
    atom_virial = torch.empty((nf, nall * 9), dtype=dt, device=dev)
    lib = L.load()
    wsb = int(lib.gbdp_prod_workspace_bytes(nf, nloc, nall, nnei, int(deterministic)))
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=dev)
    fn = getattr(lib, f"gbdp_prod_force_virial_a_{L.sfx(dt)}")
    net_deriv = net_deriv.contiguous()
    in_deriv = in_deriv.to(dt).contiguous()
    rij = rij.to(dt).contiguous()
    nlist = nlist.to(torch.int32).contiguous()
    L.check(fn(_ptr(force), _ptr(virial), _ptr(atom_virial), _ptr(net_deriv), _ptr(in_deriv),
               _ptr(rij), _ptr(nlist), nloc, nall, nnei, nf, int(deterministic), _ptr(ws),
               ctypes.c_size_t(wsb), _stream()), "prod_force_virial_se_a")
    return force, virial, atom_virial


def prod_force_grad_impl(grad, in_deriv, nlist, nloc, nnei, nf):
    dt = grad.dtype
    out = torch.empty((nf, nloc * nnei * 4), dtype=dt, device=grad.device)
    fn = getattr(L.load(), f"gbdp_prod_force_grad_a_{L.sfx(dt)}")
    grad = grad.contiguous()
    in_deriv = in_deriv.to(dt).contiguous()
    nlist = nlist.to(torch.int32).contiguous()
    L.check(fn(_ptr(out), _ptr(grad), _ptr(in_deriv), _ptr(nlist), nloc, nnei, nf, _stream()),
            "prod_force_grad_a")
    return out


def prod_virial_grad_impl(grad, in_deriv, rij, nlist, nloc, nnei, nf):
    dt = grad.dtype
    out = torch.empty((nf, nloc * nnei * 4), dtype=dt, device=grad.device)
    fn = getattr(L.load(), f"gbdp_prod_virial_grad_a_{L.sfx(dt)}")
    grad = grad.contiguous()
    in_deriv = in_deriv.to(dt).contiguous()
    rij = rij.to(dt).contiguous()
    nlist = nlist.to(torch.int32).contiguous()
    L.check(fn(_ptr(out), _ptr(grad), _ptr(in_deriv), _ptr(rij), _ptr(nlist), nloc, nnei, nf,
               _stream()), "prod_virial_grad_a")
    return out


class ProdForceFn(torch.autograd.Function):
    """force = prod_force(net_deriv); backward wrt net_deriv is prod_force_grad
    (the TF ProdForceSeA gradient, source/op/tf/prod_force_grad_multi_device.cc)."""

    @staticmethod
    def forward(ctx, net_deriv, in_deriv, nlist, natoms, n_a_sel, n_r_sel):
        ctx.save_for_backward(in_deriv, nlist)
        nat = [int(v) for v in natoms.reshape(-1).tolist()]
        ctx.dims = (nat[0], nat[1], int(n_a_sel) + int(n_r_sel), net_deriv.shape[0])
        return prod_force_se_a_impl(net_deriv, in_deriv, nlist, natoms, n_a_sel, n_r_sel)

    @staticmethod
    def backward(ctx, g_force):
        in_deriv, nlist = ctx.saved_tensors
        nloc, nall, nnei, nf = ctx.dims
        g = g_force.reshape(nf, nall, 3)[:, :nloc, :].contiguous()
        return prod_force_grad_impl(g, in_deriv, nlist, nloc, nnei, nf), None, None, None, None, None


class ProdVirialFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, net_deriv, in_deriv, rij, nlist, natoms, n_a_sel, n_r_sel):
        ctx.save_for_backward(in_deriv, rij, nlist)
        nat = [int(v) for v in natoms.reshape(-1).tolist()]
        ctx.dims = (nat[0], nat[1], int(n_a_sel) + int(n_r_sel), net_deriv.shape[0])
        return prod_virial_se_a_impl(net_deriv, in_deriv, rij, nlist, natoms, n_a_sel, n_r_sel)

    @staticmethod
    def backward(ctx, g_vir, g_atom_vir):
        in_deriv, rij, nlist = ctx.saved_tensors
        nloc, nall, nnei, nf = ctx.dims
        if g_vir is None:
            return None, None, None, None, None, None, None
        g = prod_virial_grad_impl(g_vir.contiguous(), in_deriv, rij, nlist, nloc, nnei, nf)
        return g, None, None, None, None, None, None


# -------------------------------------------------------- registration --
_REGISTERED = False
_LIBS = []


def register() -> None:
    """Define the deepmd operators in the torch dispatcher (idempotent)."""
    global _REGISTERED
    if _REGISTERED:
        return
    L.load()
    try:
        lib = torch.library.Library("deepmd", "DEF")
    except RuntimeError:
        lib = torch.library.Library("deepmd", "FRAGMENT")
    _LIBS.append(lib)

    def _def(schema, fn):
        name = schema.split("(")[0]
        if hasattr(torch.ops.deepmd, name):
            try:
                getattr(torch.ops.deepmd, name).default
                return
            except Exception:
                pass
        lib.define(schema)
        lib.impl(name, fn, "CompositeImplicitAutograd")

    _def("enable_mpi() -> Tensor", lambda: torch.zeros(1, dtype=torch.bool))
    _def("tabulate_fusion_se_a(Tensor table, Tensor table_info, Tensor em_x, Tensor em, "
         "int last_layer_size) -> Tensor[]", tabulate_fusion_se_a)
    _def("prod_env_mat_a(Tensor coord, Tensor type, Tensor natoms, Tensor box, Tensor mesh, "
         "Tensor davg, Tensor dstd, float rcut_a, float rcut_r, float rcut_r_smth, int[] sel_a, "
         "int[] sel_r) -> Tensor[]", prod_env_mat_a_impl)
    _def("prod_env_mat_a_nlist(Tensor coord, Tensor type, Tensor nlist, Tensor davg, "
         "Tensor dstd, float rcut, float rcut_smth, int[] sel) -> Tensor[]",
         prod_env_mat_a_nlist_impl)
    _def("prod_force_se_a(Tensor net_deriv, Tensor in_deriv, Tensor nlist, Tensor natoms, "
         "int n_a_sel, int n_r_sel) -> Tensor",
         lambda net_deriv, in_deriv, nlist, natoms, n_a_sel, n_r_sel: ProdForceFn.apply(
             net_deriv, in_deriv, nlist, natoms, n_a_sel, n_r_sel))
    _def("prod_virial_se_a(Tensor net_deriv, Tensor in_deriv, Tensor rij, Tensor nlist, "
         "Tensor natoms, int n_a_sel, int n_r_sel) -> Tensor[]",
         lambda net_deriv, in_deriv, rij, nlist, natoms, n_a_sel, n_r_sel: list(
             ProdVirialFn.apply(net_deriv, in_deriv, rij, nlist, natoms, n_a_sel, n_r_sel)))
    _REGISTERED = True
