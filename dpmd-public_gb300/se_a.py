"""se_e2_a energy / force / virial on GB300, three forms over one model:

* ``fused``      the chosen form: periodic neighbour build + env matrix
                 (libgbdp), fused tabulated descriptor forward (libgbdp),
                 per-type fitting nets (cuBLAS GEMMs, forward and input
                 gradient), fused descriptor backward with the force / virial
                 scatter (libgbdp).  Packed ragged batches, static buffers,
                 capturable in a CUDA graph.
* ``ops``        the compressed model through the reference's operator
                 contract: prod_env_mat_a -> torch.ops.deepmd.
                 tabulate_fusion_se_a per section -> fitting -> autograd to
                 dE/d(env) -> prod_force_se_a / prod_virial_se_a
                 (the sequence of deepmd/tf/descriptor/se_a.py:652-765).
* ``plain``      the uncompressed model: as ``ops`` but the embedding nets
                 run as matmuls (deepmd/pt/model/descriptor/se_a.py:823-845).
* ``plain-tc``   the uncompressed model with the embedding nets fused with
                 G^T R on the tensor cores (BF16 MMAs, FP32 accumulation;
                 libgbdp), forward and backward, then the force / virial
                 operators.

Energies and virials are reduced per frame in float64.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib as L
from . import model as mdl
from .ops import (EnvMatResult, NeighborPlan, VerletList, env_mat_packed, env_mat_skin,
                  prod_force_se_a_impl, prod_force_virial_se_a_impl, prod_virial_se_a_impl)

_P = ctypes.c_void_p


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


# ----------------------------------------------- tensor-core embedding --
# Per-net parameter block of the BF16 embedding kernels (csrc/embed_tc.cu):
# weight images in the shared-memory layout the MMAs read, then FP32 params.
EMB_TC_WIDTHS = ((25, 50, 100), (3, 6, 12))
_NET_B2, _NET_B3, _NET_PAR, _NET_B3T, _NET_B2T, _NET_BYTES = 0, 8192, 24576, 26624, 43008, 51200


def _bf16_bits(a: np.ndarray) -> np.ndarray:
    """FP32 -> BF16 bit patterns, rounded to nearest even."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def _sw128_image(m: np.ndarray, nrows: int) -> bytes:
    """m [n, k] as the BF16 K-major operand image with nrows rows (zero
    padded) and K in chunks of 64: chunk c holds rows of 128 bytes, and the
    16-byte piece p of row n is stored at piece p ^ (n & 7)."""
    n, k = m.shape
    nch = (k + 63) // 64
    pad = np.zeros((nrows, nch * 64), np.float32)
    pad[:n, :k] = m
    bits = _bf16_bits(pad).reshape(nrows, nch, 8, 8).transpose(1, 0, 2, 3)
    out = np.empty_like(bits)
    rows = np.arange(nrows)
    for piece in range(8):
        out[:, rows, piece ^ (rows & 7), :] = bits[:, :, piece, :]
    return out.tobytes()


def embed_tc_images(emb) -> np.ndarray:
    """[nnets, 51200] uint8: per embedding net W2^T, W3^T (forward), w1, b1,
    b2, b3 (FP32), W3, W2 (backward)."""
    out = np.zeros((len(emb), _NET_BYTES), np.uint8)
    for k, layers in enumerate(emb):
        (w1, b1), (w2, b2), (w3, b3) = [(np.asarray(l["w"], np.float32),
                                         np.asarray(l["b"], np.float32)) for l in layers]
        blk = out[k]

        def put(off, data):
            blk[off:off + len(data)] = np.frombuffer(data, np.uint8)

        put(_NET_B2, _sw128_image(w2.T, 64))
        put(_NET_B3, _sw128_image(w3.T, 128))
        par = np.zeros(320, np.float32)
        par[:w1.shape[1]] = w1[0]
        par[64:64 + len(b1)] = b1
        par[128:128 + len(b2)] = b2
        par[192:192 + len(b3)] = b3
        put(_NET_PAR, par.tobytes())
        put(_NET_B3T, _sw128_image(w3, 64))
        put(_NET_B2T, _sw128_image(w2, 64))
    return out


def _emb_tc_ok(cfg, emb) -> bool:
    """The tensor-core kernels serve 1 -> N1 -> N2 -> N3 nets of the built
    widths whose skips follow the widths (none, then identity or [x, x])."""
    if tuple(cfg.neuron) not in EMB_TC_WIDTHS:
        return False
    for net in emb:
        if len(net) != 3 or net[0]["skip"] != "none":
            return False
        for l in net[1:]:
            n_in, n_out = np.asarray(l["w"]).shape
            want = "same" if n_in == n_out else ("double" if n_out == 2 * n_in else "none")
            if l["skip"] != want:
                return False
    return True


class SeAModel:
    FIT_MODES = ("fp32", "tf32x3", "bf16", "native-fp32", "native-bf16x9", "native-tf32",
                 "native-bf16", "tc-f16x3")
    _NATIVE = {"native-fp32": 0, "native-bf16x9": 1, "native-tf32": 2, "native-bf16": 3}

    def __init__(self, cfg: mdl.SeAConfig, params: dict, davg: np.ndarray, dstd: np.ndarray,
                 device, dtype=torch.float32, tables=None, table_infos=None, fit_mode="fp32"):
        """fit_mode selects the fitting GEMMs: "fp32" (cuBLAS SGEMM),
        "tf32x3" (torch GEMMs, each operand split into a TF32 head and a
        remainder, three tensor-core products, FP32-level accuracy), "bf16"
        (BF16 tensor cores with FP32 accumulation, a stated larger error),
        "native-*" (the library's cuBLAS call with that compute type) or
        "tc-f16x3" (the library's tcgen05 kernels: scaled FP16 hi / lo
        operand pairs, three MMAs per product, FP32-level accuracy; FP32
        models with the 1600-240-240-240 fitting net)."""
        if fit_mode not in self.FIT_MODES:
            raise ValueError(f"fit_mode must be one of {self.FIT_MODES}")
        self.fit_mode = fit_mode if dtype == torch.float32 else "fp32"
        self.cfg = cfg
        self.device = torch.device(device)
        self.dtype = dtype
        T = lambda a: torch.tensor(np.asarray(a), dtype=dtype, device=self.device)
        self.emb = [[(T(l["w"]), T(l["b"]), l["skip"]) for l in net] for net in params["emb"]]
        self.fit = []
        for f in params["fit"]:
            hidden = [(T(l["w"]), T(l["b"]), None if l["idt"] is None else T(l["idt"]), l["skip"])
                      for l in f["hidden"]]
            self.fit.append((hidden, T(f["final"]["w"]), T(f["final"]["b"])))
        self.bias_atom_e = T(params["bias_atom_e"])
        self.params_bias = np.asarray(params["bias_atom_e"], np.float64)
        # transposed / split copies of the fitting weights for the GEMM modes
        self._wsplit = {}
        self._wt = {}
        for f in self.fit:
            for w, *_ in f[0]:
                wt = w.t().contiguous()
                self._wt[w.data_ptr()] = wt
                if dtype == torch.float32:
                    for mat in (w, wt):
                        self._wsplit[mat.data_ptr()] = _split_tf32(mat) + (mat.to(torch.bfloat16),)
        self.davg = T(davg).contiguous()
        self.dstd = T(dstd).contiguous()
        self.dstd_inv = T(1.0 / np.asarray(dstd)).contiguous()
        self.tables = None
        if tables is not None:
            self.tables = [T(t).contiguous() for t in tables]
            self.table_infos = np.asarray(table_infos, np.float64)
            self.table_info_t = [torch.tensor(i, dtype=dtype) for i in self.table_infos]  # CPU
            ct = ctypes.c_double if dtype == torch.float64 else ctypes.c_float
            # the fused kernels read a k-planar copy of each table
            self.tables_kp = [self._planar(t) for t in self.tables]
            self._tab_ptrs = (_P * len(self.tables_kp))(*[t.data_ptr() for t in self.tables_kp])
            flat = self.table_infos.reshape(-1)
            self._tab_infos = (ct * len(flat))(*flat.tolist())
        self._sel_c = (ctypes.c_int * cfg.ntypes)(*[int(s) for s in cfg.sel])
        # weights for the tensor-core fitting (tcgen05 kind::f16): FP16 hi / lo
        # images under per-row power-of-two scales, the matching inverse
        # column scales, and the activation scales from parameter bounds
        self._tc_nets = None
        if dtype == torch.float32 and self.fit_mode == "tc-f16x3":
            nets = (L.FitTcNet * cfg.ntypes)()
            self._tc_keep = []
            for t, (hidden, wf, bf) in enumerate(self.fit):
                if len(hidden) != 3 or [w.shape for w, *_ in hidden] != [(1600, 240), (240, 240),
                                                                           (240, 240)]:
                    raise ValueError("tc-f16x3 serves the 1600-240-240-240 fitting net only")
                if hidden[0][2] is not None or hidden[1][2] is None or hidden[2][2] is None:
                    raise ValueError("tc-f16x3 expects a time step on layers 2 and 3 only")
                wo = wf[:, 0].contiguous()
                act = _fit_tc_act_scales(hidden, wo)
                s_in = [1.0, act[0], act[1]]   # D rows carry their own scales
                s_g = [act[4], act[3], act[2]]  # GZ1, GZ2, GZ3 feed layers 0, 1, 2 back
                for l, (w, b_, idt, skip) in enumerate(hidden):
                    wth, wtl, inv_v = _split_f16_rows(w.t().contiguous())
                    wh, wl, inv_u = _split_f16_rows(w.contiguous())
                    csf = (inv_v / s_in[l]).contiguous()
                    csb = (inv_u / s_g[l]).contiguous()
                    self._tc_keep += [wh, wl, wth, wtl, csf, csb]
                    nets[t].w_hi[l], nets[t].w_lo[l] = wh.data_ptr(), wl.data_ptr()
                    nets[t].wt_hi[l], nets[t].wt_lo[l] = wth.data_ptr(), wtl.data_ptr()
                    nets[t].cs_fwd[l], nets[t].cs_bwd[l] = csf.data_ptr(), csb.data_ptr()
                    nets[t].b[l] = b_.data_ptr()
                    nets[t].idt[l] = 0 if idt is None else idt.data_ptr()
                for a in range(5):
                    nets[t].act_scale[a] = act[a]
                self._tc_keep.append(wo)
                nets[t].w_out = wo.data_ptr()
                nets[t].b_out = float(bf[0])
            self._tc_nets = nets
        # pointer tables for the native fitting entry point (float32 only)
        self._fit_c = []
        if dtype == torch.float32:
            for hidden, wf, bf in self.fit:
                nh = len(hidden)
                widths = (ctypes.c_int * (nh + 1))(cfg.dim_descrpt, *[w.shape[1] for w, *_ in hidden])
                wp = (_P * nh)(*[w.data_ptr() for w, *_ in hidden])
                bp = (_P * nh)(*[b_.data_ptr() for _, b_, *_ in hidden])
                ip = (_P * nh)(*[(0 if idt is None else idt.data_ptr()) for _, _, idt, _ in hidden])
                wout = wf[:, 0].contiguous()
                self._fit_c.append((nh, widths, wp, bp, ip, wout, float(bf[0])))
        # BF16 tensor-core embedding for the uncompressed form (FP32 models)
        self._emb_tc = None
        if dtype == torch.float32 and _emb_tc_ok(cfg, params["emb"]):
            self._emb_tc = torch.from_numpy(embed_tc_images(params["emb"])).to(self.device)
        self._sfx = L.sfx(dtype)
        self._lib = L.load()

    def _planar(self, table: torch.Tensor) -> torch.Tensor:
        lib = L.load()
        nrow, w6 = table.shape
        m = w6 // 6
        re = lib.gbdp_table_planar_row_elems(m, table.element_size())
        dst = torch.empty(nrow * re, dtype=table.dtype, device=table.device)
        if dst.data_ptr() % 128:
            raise RuntimeError("planar table allocation is not 128-byte aligned")
        stream = torch.cuda.current_stream(table.device).cuda_stream
        fn = lib.gbdp_table_to_planar_f64 if table.dtype == torch.float64 else \
            lib.gbdp_table_to_planar_f32
        L.check(fn(dst.data_ptr(), table.data_ptr(), nrow, m, stream), "table_to_planar")
        return dst

    # ------------------------------------------------------------- batches --
    def batch(self, atype_per_frame, boxes, max_cand: int = 0, skin: float = 0.0) -> "Batch":
        return Batch(self, atype_per_frame, boxes, max_cand, skin)

    # ------------------------------------------------------------ fitting --
    def _mm(self, a: torch.Tensor, w: torch.Tensor, out=None):
        """a @ w in the selected fitting mode (w is a weight matrix whose
        split copies were prepared at construction)."""
        if self.fit_mode == "fp32":
            return torch.mm(a, w, out=out)
        w_hi, w_lo, w_bf = self._wsplit[w.data_ptr()]
        if self.fit_mode == "bf16":
            r = torch.mm(a.to(torch.bfloat16), w_bf).to(torch.float32)
            if out is not None:
                out.copy_(r)
                return out
            return r
        a_hi, a_lo = _split_tf32(a)
        prev = torch.backends.cuda.matmul.allow_tf32
        torch.backends.cuda.matmul.allow_tf32 = True
        try:
            r = torch.mm(a_hi, w_hi, out=out)
            r.addmm_(a_hi, w_lo)
            r.addmm_(a_lo, w_hi)
        finally:
            torch.backends.cuda.matmul.allow_tf32 = prev
        return r

    def fitting_fwd_bwd(self, t: int, D: torch.Tensor, dD_out=None):
        """Energy of type-t atoms and dE/dD (hidden tanh layers with idt /
        skip where present, linear output; deepmd/pt/model/task/fitting.py
        with deepmd/dpmodel/utils/network.py layer semantics).  dE/dD is
        written into ``dD_out`` when given."""
        hidden, wf, bf = self.fit[t]
        h = D
        cache = []
        for w, b, idt, skip in hidden:
            tt = torch.tanh(self._mm(h, w).add_(b))
            out = tt * idt if idt is not None else tt
            if skip == "same":
                out = out + h
            cache.append((tt, idt, skip, w))
            h = out
        e = torch.addmm(bf, h, wf)[:, 0] + self.bias_atom_e[t]
        g = wf[:, 0].expand(h.shape[0], -1)
        for k, (tt, idt, skip, w) in enumerate(reversed(cache)):
            gt = g * idt if idt is not None else g
            gz = gt * (1 - tt * tt)
            last = k == len(cache) - 1
            gin = self._mm(gz, self._wt[w.data_ptr()], out=dD_out if (last and skip != "same") else None)
            if skip == "same":
                gin = gin + g
                if last and dD_out is not None:
                    dD_out.copy_(gin)
            g = gin
        return e, g

    def fitting_energy(self, t: int, D: torch.Tensor):
        hidden, wf, bf = self.fit[t]
        h = D
        for w, b, idt, skip in hidden:
            tt = torch.tanh(torch.addmm(b, h, w))
            out = tt * idt if idt is not None else tt
            if skip == "same":
                out = out + h
            h = out
        return torch.addmm(bf, h, wf)[:, 0] + self.bias_atom_e[t]

    # ------------------------------------------------------- chosen form --
    def step_fused(self, b: "Batch", coord: torch.Tensor, deterministic: bool | None = None,
                   rebuild: bool = True):
        """E [nframes] f64, F [nloc_total, 3], virial [nframes, 9] f64.
        deterministic: forces, virials and energies summed in 64-bit fixed
        point, the same bits on every run (floating-point atomics otherwise).
        Default: on for FP32 models (its 2^-32 eV/A grid is far below FP32
        rounding, and the integer sums measured faster than the FP64
        atomics of the frame virial), off for FP64 models (whose rounding is
        finer than the 2^-40 grid).
        rebuild: for a batch made with a skin, rebuild the Verlet list (and
        ghosts) at this step; otherwise the list of the last rebuild is
        reused with the ghosts following their atoms.  A batch without a
        skin rebuilds at every step."""
        if deterministic is None:
            deterministic = self.dtype == torch.float32
        cfg = self.cfg
        if self.tables is None:
            raise RuntimeError("the fused form needs the compression tables")
        M, A = cfg.neuron[-1], cfg.axis_neuron
        n = b.nloc
        if b.skin > 0:
            env_mat_skin(b.plan, b.vl, coord, b.atype, self.davg, self.dstd, cfg.rcut,
                         cfg.rcut_smth, list(cfg.sel), rebuild, out=b.env)
        else:
            env_mat_packed(b.plan, coord, b.atype, self.davg, self.dstd, cfg.rcut_smth,
                           list(cfg.sel), check_status=False, out=b.env)
        lib = self._lib
        if self._tc_nets is not None:
            L.check(lib.gbdp_se_a_descriptor_fwd_split_f32(
                _ptr(b.X), _ptr(b.D), _ptr(b.D_lo), _ptr(b.D_rs), _ptr(b.env.em), _ptr(b.atype),
                _ptr(b.drow),
                self._tab_ptrs, self._tab_infos, cfg.ntypes, self._sel_c, int(cfg.type_one_side), n,
                M, A, _stream()), "se_a_descriptor_fwd_split")
            self.fitting_tc(b)
        else:
            L.check(getattr(lib, f"gbdp_se_a_descriptor_fwd_{self._sfx}")(
                _ptr(b.X), _ptr(b.D), _ptr(b.env.em), _ptr(b.atype), _ptr(b.drow), self._tab_ptrs,
                self._tab_infos, cfg.ntypes, self._sel_c, int(cfg.type_one_side), n, M, A,
                _stream()), "se_a_descriptor_fwd")
            self.fitting_rows(b)
        L.check(getattr(lib, f"gbdp_se_a_descriptor_bwd_{self._sfx}")(
            _ptr(b.force), _ptr(b.vir), _ptr(b.X), _ptr(b.dD), _ptr(b.drow), _ptr(b.env.em),
            _ptr(b.env.nlist_ext),
            _ptr(b.env.ext_coord), _ptr(b.env.ext_map), _ptr(b.atype), _ptr(self.dstd_inv),
            _ptr(b.atom_frame), _ptr(b.frame_aoff), _ptr(b.frame_eoff), self._tab_ptrs,
            self._tab_infos, cfg.ntypes, self._sel_c, int(cfg.type_one_side),
            ctypes.c_float(cfg.rcut_smth), ctypes.c_float(cfg.rcut), n, b.nframes, M, A,
            _ptr(b.force_fx() if deterministic else None), _stream()), "se_a_descriptor_bwd")
        L.check(getattr(lib, f"gbdp_frame_energy_{self._sfx}")(
            _ptr(b.energy), _ptr(b.ae), _ptr(b.frame_of_row), b.ae.numel(), b.nframes,
            int(deterministic), _stream()), "frame_energy")
        return b.energy, b.force, b.vir

    def fitting_tc(self, b: "Batch"):
        """Both types' fitting nets on the tensor cores (six tcgen05 GEMM
        launches with fused epilogues over the padded type blocks)."""
        nt = self.cfg.ntypes
        nrows = (ctypes.c_int * nt)(*[c for _, c in b.type_rows])
        L.check(self._lib.gbdp_fitting_tc_f32(
            _ptr(b.ae), _ptr(b.dD), _ptr(b.D), _ptr(b.D_lo), _ptr(b.D_rs), nt, nrows, b.row_off_c,
            self._tc_nets,
            _ptr(b.tc_ws), ctypes.c_size_t(b.tc_ws.numel()), _stream()), "fitting_tc")
        for t, (s0, cnt) in enumerate(b.type_rows):
            if cnt and float(self.params_bias[t]) != 0.0:
                b.ae[s0:s0 + cnt].add_(float(self.params_bias[t]))

    def fitting_rows(self, b: "Batch"):
        """Per-type fitting over the type-contiguous rows of D (each atom
        through its own type's net only)."""
        native = self._NATIVE.get(self.fit_mode)
        for t, (s0, nt) in enumerate(b.type_rows):
            if nt == 0:
                continue
            if native is None:
                e, _ = self.fitting_fwd_bwd(t, b.D[s0:s0 + nt], dD_out=b.dD[s0:s0 + nt])
                b.ae[s0:s0 + nt].copy_(e)
                continue
            nh, widths, wp, bp, ip, wout, bout = self._fit_c[t]
            ws = b.fit_ws(t, self)
            L.check(self._lib.gbdp_fitting_fwd_bwd_f32(
                _ptr(b.ae[s0:s0 + nt]), _ptr(b.dD[s0:s0 + nt]), _ptr(b.D[s0:s0 + nt]), nt, widths,
                nh, wp, bp, ip, _ptr(wout), ctypes.c_float(bout), native, _ptr(ws),
                ctypes.c_size_t(ws.numel()), _stream()), "fitting_fwd_bwd")
            if float(self.params_bias[t]) != 0.0:
                b.ae[s0:s0 + nt].add_(self.params_bias[t])

    def embed_tc_forward(self, b: "Batch", em: torch.Tensor):
        """X [nloc, 4, M] and D (rows of b) of the uncompressed descriptor
        from the env matrix, embedding on the tensor cores (BF16)."""
        if self._emb_tc is None:
            raise RuntimeError("the tensor-core embedding serves FP32 models with embedding "
                               f"widths {EMB_TC_WIDTHS}")
        cfg = self.cfg
        n1, n2, n3 = cfg.neuron
        sel = (ctypes.c_int * cfg.ntypes)(*[int(x) for x in cfg.sel])
        L.check(self._lib.gbdp_embed_fwd_tc_bf16(
            _ptr(b.X), _ptr(b.D), _ptr(getattr(b, "D_lo", None)), _ptr(getattr(b, "D_rs", None)),
            _ptr(b.drow), _ptr(em),
            _ptr(b.atype), _ptr(b.units), b.nunits, _ptr(self._emb_tc), cfg.ntypes, sel,
            int(cfg.type_one_side), b.nloc, cfg.nnei, n1, n2, n3, cfg.axis_neuron,
            _ptr(b.emb_status), _stream()), "embed_fwd_tc")

    def embed_tc_backward(self, b: "Batch", em: torch.Tensor) -> torch.Tensor:
        """dE/d(env matrix) [nloc, nnei, 4] from b.dD (the fitting's dE/dD)."""
        cfg = self.cfg
        n1, n2, n3 = cfg.neuron
        sel = (ctypes.c_int * cfg.ntypes)(*[int(x) for x in cfg.sel])
        L.check(self._lib.gbdp_embed_bwd_tc_bf16(
            _ptr(b.net_deriv), _ptr(b.dx_work), _ptr(b.dD), _ptr(b.X), _ptr(b.drow), _ptr(em),
            _ptr(b.atype), _ptr(b.units), b.nunits, _ptr(self._emb_tc), cfg.ntypes, sel,
            int(cfg.type_one_side), b.nloc, cfg.nnei, n1, n2, n3, cfg.axis_neuron,
            _ptr(b.emb_status), _stream()), "embed_bwd_tc")
        return b.net_deriv

    def step_plain_tc(self, b: "Batch", coord: torch.Tensor):
        """The uncompressed model on the GPU with the embedding nets on the
        tensor cores: env matrix (with derivatives) -> fused embedding +
        G^T R + D (BF16 MMAs) -> fitting -> fused embedding backward ->
        prod_force_se_a / prod_virial_se_a per frame.  E [nframes] f64,
        F [nloc_total, 3], virial [nframes, 9] f64."""
        cfg = self.cfg
        nnei = cfg.nnei
        b.ensure_plain_tc(self)
        env = env_mat_packed(b.plan, coord, b.atype, self.davg, self.dstd, cfg.rcut_smth,
                             list(cfg.sel), check_status=False, out=b.env_full)
        self.embed_tc_forward(b, env.em)
        if self._tc_nets is not None:
            self.fitting_tc(b)
        else:
            self.fitting_rows(b)
        net = self.embed_tc_backward(b, env.em)
        forces, virs = [], []
        for f in range(b.nframes):
            a0, nl = int(b.plan.atom_off[f]), int(b.plan.nloc[f])
            natoms = torch.tensor([nl, nl] + [0] * cfg.ntypes, dtype=torch.int32)
            nd = net[a0:a0 + nl].reshape(1, -1)
            ed = env.em_deriv[a0:a0 + nl].reshape(1, -1)
            nlst = env.nlist[a0:a0 + nl].reshape(1, -1)
            f_, v, _ = prod_force_virial_se_a_impl(nd, ed, env.rij[a0:a0 + nl].reshape(1, -1),
                                                   nlst, natoms, nnei, 0)
            forces.append(f_.reshape(nl, 3))
            virs.append(v.reshape(9))
        L.check(getattr(self._lib, f"gbdp_frame_energy_{self._sfx}")(
            _ptr(b.energy), _ptr(b.ae), _ptr(b.frame_of_row), b.ae.numel(), b.nframes, 0,
            _stream()), "frame_energy")
        return b.energy, torch.cat(forces), torch.stack(virs).to(torch.float64)

    # --------------------------------------------- operator-contract forms --
    def _descriptor_from_em(self, em: torch.Tensor, atype: torch.Tensor, compressed: bool):
        cfg = self.cfg
        n = em.shape[0]
        sec = cfg.sec
        M, A = cfg.neuron[-1], cfg.axis_neuron
        X = torch.zeros((n, 4, M), dtype=self.dtype, device=self.device)
        for tj in range(cfg.ntypes):
            centres = [None] if cfg.type_one_side else list(range(cfg.ntypes))
            for ti in centres:
                k = tj if cfg.type_one_side else tj * cfg.ntypes + ti
                rows = None if ti is None else torch.nonzero(atype == ti).reshape(-1)
                rr = em[:, sec[tj]:sec[tj + 1], :] if rows is None else em[rows, sec[tj]:sec[tj + 1], :]
                if rr.shape[0] == 0 or rr.shape[1] == 0:
                    continue
                ss = rr[:, :, :1]
                if compressed:
                    gr = torch.ops.deepmd.tabulate_fusion_se_a(
                        self.tables[k], self.table_info_t[k], ss.reshape(-1, 1).contiguous(),
                        rr.contiguous(), M)[0]
                else:
                    gg = ss
                    for w, b_, skip in self.emb[k]:
                        y = torch.tanh(torch.matmul(gg, w) + b_)
                        if skip == "same":
                            y = y + gg
                        elif skip == "double":
                            y = y + torch.cat([gg, gg], -1)
                        gg = y
                    gr = torch.matmul(rr.permute(0, 2, 1), gg)
                X = X + gr if rows is None else X.index_add(0, rows, gr)
        X = X / cfg.nnei
        return torch.matmul(X.permute(0, 2, 1), X[:, :, :A]).reshape(n, M * A)

    def step_ops(self, b: "Batch", coord: torch.Tensor, compressed: bool = True,
                 deterministic: bool = False):
        """The drop-in sequence through the operator contract, frame by frame
        of the batch (the reference processes one frame at a time)."""
        cfg = self.cfg
        nnei = cfg.nnei
        env = env_mat_packed(b.plan, coord, b.atype, self.davg, self.dstd, cfg.rcut_smth,
                             list(cfg.sel), need_deriv=True, need_rij=True, check_status=False)
        em = env.em.detach().requires_grad_(True)
        D = self._descriptor_from_em(em, b.atype, compressed)
        E_atom = torch.zeros(b.nloc, dtype=self.dtype, device=self.device)
        for t in range(cfg.ntypes):
            idx = b.type_idx[t]
            if idx.numel():
                E_atom = E_atom.index_add(0, idx, self.fitting_energy(t, D.index_select(0, idx)))
        net = torch.autograd.grad(E_atom.sum(), em)[0]
        forces, virs = [], []
        for f in range(b.nframes):
            a0, a1 = int(b.plan.atom_off[f]), int(b.plan.atom_off[f]) + int(b.plan.nloc[f])
            nl = int(b.plan.nloc[f])
            natoms = torch.tensor([nl, nl] + [0] * cfg.ntypes, dtype=torch.int32)
            nd = net[a0:a1].reshape(1, -1)
            ed = env.em_deriv[a0:a1].reshape(1, -1)
            nlst = env.nlist[a0:a1].reshape(1, -1)
            f_, v, _ = prod_force_virial_se_a_impl(nd, ed, env.rij[a0:a1].reshape(1, -1), nlst,
                                                   natoms, nnei, 0, deterministic)
            forces.append(f_.reshape(nl, 3))
            virs.append(v.reshape(9))
        E = torch.zeros(b.nframes, dtype=torch.float64, device=self.device)
        E.index_add_(0, b.frame_of_atom, E_atom.detach().to(torch.float64))
        return E, torch.cat(forces), torch.stack(virs).to(torch.float64)


    def step_lower(self, ext_coord: torch.Tensor, ext_atype: torch.Tensor,
                   nlist: torch.Tensor, mapping: torch.Tensor, nloc: int,
                   compressed: bool = True):
        """The forward_lower path of one frame (deepmd/pt/model/model/
        make_model.py:334-415, called by DeepPotPT::compute): extended
        coordinates [nall, 3] with the local atoms first, extended types,
        an external neighbour list [nloc, nnei_in] (unsorted, rcut + skin)
        and the extended -> local mapping.  Env matrix through
        prod_env_mat_a_nlist, descriptor and fitting as the operator form,
        forces on the extended atoms folded back to the local ones through
        the mapping (communicate_extended_output,
        deepmd/pt/model/model/transform_output.py:317-380).
        Returns E (FP64 scalar), F [nloc, 3], virial [9] (FP64)."""
        cfg = self.cfg
        nnei = cfg.nnei
        nall = ext_atype.numel()
        em, emd, rij, nl = torch.ops.deepmd.prod_env_mat_a_nlist(
            ext_coord.reshape(1, -1), ext_atype.reshape(1, -1), nlist.reshape(1, nloc, -1),
            self.davg, self.dstd, cfg.rcut, cfg.rcut_smth, list(cfg.sel))
        em = em.reshape(nloc, nnei, 4).detach().requires_grad_(True)
        atype = ext_atype[:nloc].to(torch.int32)
        D = self._descriptor_from_em(em, atype, compressed)
        E_atom = torch.zeros(nloc, dtype=self.dtype, device=self.device)
        for t in range(cfg.ntypes):
            idx = torch.nonzero(atype == t).reshape(-1)
            if idx.numel():
                E_atom = E_atom.index_add(0, idx, self.fitting_energy(t, D.index_select(0, idx)))
        net = torch.autograd.grad(E_atom.sum(), em)[0].reshape(1, -1)
        natoms = torch.tensor([nloc, nall] + [0] * cfg.ntypes, dtype=torch.int32)
        f_ext = prod_force_se_a_impl(net, emd, nl, natoms, nnei, 0).reshape(nall, 3)
        vir, _ = prod_virial_se_a_impl(net, emd, rij, nl, natoms, nnei, 0)
        F = torch.zeros((nloc, 3), dtype=self.dtype, device=self.device)
        F.index_add_(0, mapping.to(torch.int64), f_ext)
        return E_atom.detach().to(torch.float64).sum(), F, vir.reshape(9).to(torch.float64)


def _rn_tf32(x: torch.Tensor) -> torch.Tensor:
    """x rounded to TF32 (10 explicit mantissa bits): to nearest, ties away
    from zero, on the magnitude bits of the FP32 pattern."""
    return ((x.contiguous().view(torch.int32) + 0x1000) & -8192).view(torch.float32)


def _split_tf32(x: torch.Tensor):
    """x ~= hi + lo, hi = x rounded to TF32 and lo = (x - hi) rounded to
    TF32, so that both are exact tensor-core operands and
    |x - hi - lo| <= 2^-23 |x|."""
    hi = _rn_tf32(x)
    return hi, _rn_tf32(x - hi)


def _f16_scale(bound: float) -> float:
    """2^s with bound * 2^s < 2^15 (1 for a zero or non-finite bound): the
    power-of-two scale under which a block with magnitudes up to ``bound``
    splits into FP16 hi / lo parts without overflow."""
    if not (bound > 0.0) or not math.isfinite(bound):
        return 1.0
    return math.ldexp(1.0, 15 - max(math.frexp(bound)[1], -100))


def _split_f16_rows(m: torch.Tensor):
    """FP16 hi / lo images of m [rows, K] (FP32), row r scaled by 2^u_r
    (``_f16_scale`` of the row's largest magnitude): hi = fp16(m 2^u),
    lo = fp16(m 2^u - hi), both rounded to nearest; and 2^-u [rows]."""
    mx = m.abs().amax(dim=1).double().cpu().numpy()
    sc = torch.tensor([_f16_scale(float(v)) for v in mx], dtype=torch.float32, device=m.device)
    x = m * sc[:, None]
    hi = x.half()
    lo = (x - hi.float()).half()
    return hi.contiguous(), lo.contiguous(), 1.0 / sc


def _fit_tc_act_scales(hidden, wo: torch.Tensor) -> list:
    """Scales of the tensor-core fitting's split activations H1, H2, GZ3,
    GZ2, GZ1 of one net, from bounds on their magnitudes over any input:
    |T| <= 1 and 0 <= 1 - T^2 <= 1 for every tanh output T, and
    |sum_j g_j W_ij| <= max|g| max_i sum_j |W_ij| for every GEMM (1 %
    margin for FP32 rounding)."""
    (_, _, _, _), (w2, _, idt2, _), (w3, _, idt3, _) = hidden
    f = lambda x: float(x.double().abs().max())
    rows = lambda w: float(w.double().abs().sum(dim=1).max())
    b_h1 = 1.0
    b_h2 = 1.0 + f(idt2)
    b_gz3 = f(wo.double() * idt3.double())
    b_g2 = b_gz3 * rows(w3) + f(wo)
    b_gz2 = b_g2 * f(idt2)
    b_gz1 = b_gz2 * rows(w2) + b_g2
    return [_f16_scale(1.01 * b) for b in (b_h1, b_h2, b_gz3, b_gz2, b_gz1)]


def energy_std_loss(E, F, V, E_ref, F_ref, V_ref, natoms: int, pref_e=0.02, pref_f=1000.0,
                    pref_v=0.02):
    """EnergyStdLoss with fixed prefactors (deepmd/pt/loss/ener.py:197-360):
    pref_e * mean((E - E_ref)^2) / natoms^2 ... as the reference scales the
    energy and virial terms by 1/natoms (atom_norm), plus pref_f * mean of the
    squared force error."""
    inv = 1.0 / natoms
    l_e = ((E - E_ref) ** 2).mean() * inv * inv
    l_f = ((F - F_ref) ** 2).mean()
    l_v = ((V - V_ref) ** 2).mean() * inv * inv
    return pref_e * l_e + pref_f * l_f + pref_v * l_v


class Trainable:
    """Fitting-net parameters of a compressed model as autograd leaves, and
    a training forward that keeps the graph through the force (double
    backward: tabulate grad-grad, prod_force_grad / prod_virial_grad).

    gemm: "fp32" runs the fitting GEMMs in the model's dtype; "bf16" casts
    both operands of every fitting GEMM to BF16 (cuBLAS tensor-core GEMM,
    FP32 accumulation, product rounded to BF16, then back to the model's
    dtype), in the forward and in every backward order; the table path
    stays in the model's dtype."""

    GEMMS = ("fp32", "bf16")

    def __init__(self, model: SeAModel, gemm: str = "fp32"):
        if gemm not in self.GEMMS:
            raise ValueError(f"gemm must be one of {self.GEMMS}")
        self.gemm = gemm
        self.model = model
        self.params = []
        fit = []
        for hidden, wf, bf in model.fit:
            h = []
            for w, b, idt, skip in hidden:
                w = w.clone().requires_grad_(True)
                b = b.clone().requires_grad_(True)
                idt = None if idt is None else idt.clone().requires_grad_(True)
                self.params += [w, b] + ([idt] if idt is not None else [])
                h.append((w, b, idt, skip))
            wf = wf.clone().requires_grad_(True)
            bf = bf.clone().requires_grad_(True)
            self.params += [wf, bf]
            fit.append((h, wf, bf))
        self.fit = fit

    def _mm(self, a: torch.Tensor, w: torch.Tensor) -> torch.Tensor:
        if self.gemm == "bf16":
            return torch.matmul(a.to(torch.bfloat16), w.to(torch.bfloat16)).to(a.dtype)
        return a @ w

    def energy_force_virial(self, b: "Batch", coord, compressed: bool = True):
        m = self.model
        cfg = m.cfg
        nnei = cfg.nnei
        env = env_mat_packed(b.plan, coord, b.atype, m.davg, m.dstd, cfg.rcut_smth, list(cfg.sel),
                             need_deriv=True, need_rij=True, check_status=False)
        em = env.em.detach().requires_grad_(True)
        D = m._descriptor_from_em(em, b.atype, compressed)
        E_atom = torch.zeros(b.nloc, dtype=m.dtype, device=m.device)
        for t in range(cfg.ntypes):
            idx = b.type_idx[t]
            if idx.numel() == 0:
                continue
            hidden, wf, bf = self.fit[t]
            h = D.index_select(0, idx)
            for w, bb, idt, skip in hidden:
                tt = torch.tanh(self._mm(h, w) + bb)
                out = tt * idt if idt is not None else tt
                h = out + h if skip == "same" else out
            E_atom = E_atom.index_add(0, idx, (self._mm(h, wf) + bf)[:, 0] + m.bias_atom_e[t])
        net = torch.autograd.grad(E_atom.sum(), em, create_graph=True)[0]
        from .ops import ProdForceFn, ProdVirialFn

        F, V = [], []
        for f in range(b.nframes):
            a0 = int(b.plan.atom_off[f])
            nl = int(b.plan.nloc[f])
            natoms = torch.tensor([nl, nl] + [0] * cfg.ntypes, dtype=torch.int32)
            nd = net[a0:a0 + nl].reshape(1, -1)
            ed = env.em_deriv[a0:a0 + nl].reshape(1, -1)
            nls = env.nlist[a0:a0 + nl].reshape(1, -1)
            F.append(ProdForceFn.apply(nd, ed, nls, natoms, nnei, 0).reshape(nl, 3))
            V.append(ProdVirialFn.apply(nd, ed, env.rij[a0:a0 + nl].reshape(1, -1), nls, natoms, nnei,
                                        0)[0].reshape(9))
        E = torch.zeros(b.nframes, dtype=m.dtype, device=m.device).index_add(0, b.frame_of_atom, E_atom)
        return E, torch.cat(F), torch.stack(V)


class Batch:
    """Static per-batch state: the neighbour plan, type groups and every
    buffer the fused step writes (fixed addresses, so the step can be
    captured in a CUDA graph)."""

    def __init__(self, model: SeAModel, atype_per_frame, boxes, max_cand: int = 0,
                 skin: float = 0.0):
        """skin > 0: the neighbour search covers rcut + skin and keeps a
        Verlet list, which steps reuse between rebuilds (step_fused's
        ``rebuild``)."""
        cfg = model.cfg
        dev = model.device
        dt = model.dtype
        at = [np.asarray(a, np.int32).reshape(-1) for a in atype_per_frame]
        # every atom gets a row of D / dE/dD by its type, which the fused
        # kernels write and read; a type outside the model has none
        for f, a in enumerate(at):
            if a.size and (a.min() < 0 or a.max() >= cfg.ntypes):
                raise ValueError(f"frame {f}: atom types must lie in [0, {cfg.ntypes}) "
                                 f"(got {int(a.min())} .. {int(a.max())})")
        self.nframes = len(at)
        self.skin = float(skin)
        self.plan = NeighborPlan([len(a) for a in at], np.asarray(boxes, np.float64).reshape(-1, 9),
                                 cfg.rcut + self.skin, dev, dt, max_cand=max_cand)
        self.vl = VerletList(self.plan) if self.skin > 0 else None
        self.nloc = int(self.plan.nloc_total)
        flat = np.concatenate(at)
        self.atype = torch.tensor(flat, dtype=torch.int32, device=dev)
        fo = np.repeat(np.arange(self.nframes), [len(a) for a in at])
        self.frame_of_atom = torch.tensor(fo, dtype=torch.int64, device=dev)
        self.atom_frame = torch.tensor(fo, dtype=torch.int32, device=dev)
        self.frame_aoff = torch.tensor(self.plan.atom_off, dtype=torch.int32, device=dev)
        self.frame_eoff = torch.tensor(self.plan.ext_off, dtype=torch.int32, device=dev)
        self.type_idx = [torch.tensor(np.nonzero(flat == t)[0], dtype=torch.int64, device=dev)
                         for t in range(cfg.ntypes)]
        # rows of D / dE/dD grouped by type (stable within a type); the
        # tensor-core fitting pads each type's block to a multiple of 128
        pad = 128 if getattr(model, "_tc_nets", None) is not None else 1
        counts = [int((flat == t).sum()) for t in range(cfg.ntypes)]
        starts, s0 = [], 0
        for c0 in counts:
            starts.append(s0)
            s0 += -(-c0 // pad) * pad
        self.nrows_total = s0
        self.type_rows = [(int(a), int(c0)) for a, c0 in zip(starts, counts)]
        self.row_off_c = (ctypes.c_int * (cfg.ntypes + 1))(*(starts + [s0]))
        drow = np.empty(len(flat), np.int64)
        fo_row = np.full(s0, -1, np.int32)  # -1: padding row
        for t in range(cfg.ntypes):
            idx = np.nonzero(flat == t)[0]
            drow[idx] = starts[t] + np.arange(len(idx))
            fo_row[starts[t]:starts[t] + len(idx)] = fo[idx]
        self.drow = torch.tensor(drow, dtype=torch.int32, device=dev)
        self.frame_of_row = torch.tensor(fo_row, dtype=torch.int32, device=dev)
        n = self.nloc
        nnei = cfg.nnei
        M, A = cfg.neuron[-1], cfg.axis_neuron
        e = EnvMatResult()
        e.em = torch.empty((n, nnei, 4), dtype=dt, device=dev)
        e.em_deriv = None
        e.rij = None
        e.nlist = torch.empty((n, nnei), dtype=torch.int32, device=dev)
        e.nlist_ext = torch.empty((n, nnei), dtype=torch.int32, device=dev)
        e.ext_coord = torch.empty((self.plan.ext_total, 3), dtype=dt, device=dev)
        e.ext_type = torch.empty((self.plan.ext_total,), dtype=torch.int32, device=dev)
        e.ext_map = torch.empty((self.plan.ext_total,), dtype=torch.int32, device=dev)
        e.ext_nall = torch.empty((self.nframes,), dtype=torch.int32, device=dev)
        self.env = e
        self.X = torch.empty((n, 4, M), dtype=dt, device=dev)
        nr = self.nrows_total
        self.dD = torch.zeros((nr, M * A), dtype=dt, device=dev)
        self.ae = torch.zeros((nr,), dtype=dt, device=dev)
        if pad > 1:
            # D split for the tensor-core fitting: FP16 hi / lo parts of each
            # row under its power-of-two scale, and the inverse scales
            # (padding rows: zeros under scale 1)
            self.D = torch.zeros((nr, M * A), dtype=torch.float16, device=dev)
            self.D_lo = torch.zeros((nr, M * A), dtype=torch.float16, device=dev)
            self.D_rs = torch.ones((nr,), dtype=torch.float32, device=dev)
            tcb = int(model._lib.gbdp_fitting_tc_workspace_bytes(nr))
            self.tc_ws = torch.zeros(tcb, dtype=torch.uint8, device=dev)
        else:
            self.D = torch.zeros((nr, M * A), dtype=dt, device=dev)
        # the step's outputs in one device buffer (energies and virials FP64,
        # then forces), so that a caller reads them back with a single copy:
        # `out` is that buffer, energy / vir / force are views into it
        nf = self.nframes
        esz = np.dtype(np.float64).itemsize
        fbytes = n * 3 * torch.tensor([], dtype=dt).element_size()
        self.out = torch.empty(nf * 10 * esz + fbytes, dtype=torch.uint8, device=dev)
        self.energy = self.out[:nf * esz].view(torch.float64)
        self.vir = self.out[nf * esz:nf * 10 * esz].view(torch.float64).view(nf, 9)
        self.force = self.out[nf * 10 * esz:].view(dt).view(n, 3)

    def descriptor_rows(self) -> torch.Tensor:
        """D [nrows, M * axis_neuron] in the model's dtype, from the split
        FP16 parts and row scales where the tensor-core fitting is used."""
        if hasattr(self, "D_lo"):
            return (self.D.float() + self.D_lo.float()) * self.D_rs[:, None]
        return self.D

    def ensure_plain_tc(self, model: SeAModel):
        """Buffers of the tensor-core plain form (allocated once): atom pairs
        of one centre type, the full env matrix with derivatives, dE/d(env)
        and the embedding kernels' scratch and status."""
        if hasattr(self, "units"):
            return
        cfg = model.cfg
        dev = self.atype.device
        flat = self.atype.cpu().numpy()
        pairs = []
        for t in range(cfg.ntypes):
            idx = np.nonzero(flat == t)[0]
            for k in range(0, len(idx), 2):
                pairs.append((idx[k], idx[k + 1] if k + 1 < len(idx) else -1))
        self.nunits = len(pairs)
        self.units = torch.tensor(np.asarray(pairs, np.int32).reshape(-1, 2), device=dev)
        n, nnei, dt = self.nloc, cfg.nnei, model.dtype
        e = EnvMatResult()
        e.em = torch.empty((n, nnei, 4), dtype=dt, device=dev)
        e.em_deriv = torch.empty((n, nnei, 4, 3), dtype=dt, device=dev)
        e.rij = torch.empty((n, nnei, 3), dtype=dt, device=dev)
        e.nlist = torch.empty((n, nnei), dtype=torch.int32, device=dev)
        e.nlist_ext = None
        e.ext_coord = torch.empty((self.plan.ext_total, 3), dtype=dt, device=dev)
        e.ext_type = torch.empty((self.plan.ext_total,), dtype=torch.int32, device=dev)
        e.ext_map = torch.empty((self.plan.ext_total,), dtype=torch.int32, device=dev)
        e.ext_nall = torch.empty((self.nframes,), dtype=torch.int32, device=dev)
        self.env_full = e
        self.net_deriv = torch.empty((n, nnei, 4), dtype=dt, device=dev)
        self.dx_work = torch.empty((n, 4, cfg.neuron[-1]), dtype=dt, device=dev)
        self.emb_status = torch.zeros(1, dtype=torch.int32, device=dev)

    def force_fx(self) -> torch.Tensor:
        """The fixed-point force accumulator of the deterministic fused step
        (allocated once)."""
        if not hasattr(self, "_force_fx"):
            self._force_fx = torch.empty((self.nloc, 3), dtype=torch.int64, device=self.atype.device)
        return self._force_fx

    def fit_ws(self, t: int, model: SeAModel):
        """Workspace of the native fitting call for type t (allocated once)."""
        if not hasattr(self, "_fit_ws"):
            self._fit_ws = {}
        ws = self._fit_ws.get(t)
        if ws is None:
            nh, widths, wp, bp, ip, wout, bout = model._fit_c[t]
            nbytes = int(model._lib.gbdp_fitting_workspace_bytes(self.type_rows[t][1], widths, nh, ip))
            ws = torch.empty(nbytes, dtype=torch.uint8, device=self.atype.device)
            self._fit_ws[t] = ws
        return ws

    def status(self) -> int:
        """Device status word of the last neighbour build (0 = ok)."""
        return L.load().gbdp_env_status(_ptr(self.plan.workspace), _stream())


class CapturedStep:
    """The chosen form's step for one batch, captured once in a CUDA graph.

    ``replay()`` runs the step on the coordinates already in ``coord`` (a
    device buffer); calling the object with host coordinates [nloc_total, 3]
    copies them in, replays the graph and copies the packed outputs back
    into one pinned host buffer, returning host views (E [nframes] f64,
    F [nloc_total, 3], virial [nframes, 9] f64) that stay valid until the
    next call.  The graph reads and writes fixed buffers, so the batch and
    the model must outlive this object."""

    def __init__(self, model: SeAModel, b: "Batch", coord=None, warmup: int = 3,
                 deterministic=None):
        """coord: the coordinates the warm-up steps run on (host array or
        tensor, [nloc_total, 3]); later calls bring their own."""
        self.model, self.batch = model, b
        self.deterministic = deterministic
        dev = model.device
        self.coord = torch.zeros((b.nloc, 3), dtype=model.dtype, device=dev)
        if coord is not None:
            if not isinstance(coord, torch.Tensor):
                coord = torch.from_numpy(np.ascontiguousarray(coord))
            self.coord.copy_(coord.reshape(-1, 3))
        self._capture(warmup)
        self.h_coord = torch.empty((b.nloc, 3), dtype=model.dtype).pin_memory()
        self.h_out = torch.empty(b.out.numel(), dtype=torch.uint8).pin_memory()
        nf = b.nframes
        esz = 8
        self.h_energy = self.h_out[:nf * esz].view(torch.float64)
        self.h_vir = self.h_out[nf * esz:nf * 10 * esz].view(torch.float64).view(nf, 9)
        self.h_force = self.h_out[nf * 10 * esz:].view(model.dtype).view(b.nloc, 3)

    def _capture(self, warmup: int):
        model, b, deterministic = self.model, self.batch, self.deterministic
        dev = model.device
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            for _ in range(max(1, warmup)):
                model.step_fused(b, self.coord, deterministic)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        try:
            self.graph = torch.cuda.CUDAGraph(keep_graph=True)
        except TypeError:  # torch builds without keep_graph
            self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            model.step_fused(b, self.coord, deterministic)
        if hasattr(self.graph, "instantiate"):
            try:
                self.graph.instantiate()
            except RuntimeError:
                pass

    def replay(self):
        self.graph.replay()

    def h2d(self, host_coord):
        """Stage host coordinates (numpy or a CPU tensor) through the pinned
        buffer and enqueue their copy to the device."""
        if not isinstance(host_coord, torch.Tensor):
            host_coord = torch.from_numpy(np.ascontiguousarray(host_coord))
        if host_coord.data_ptr() != self.h_coord.data_ptr():
            self.h_coord.copy_(host_coord.reshape(-1, 3))
        self.coord.copy_(self.h_coord, non_blocking=True)

    def d2h(self):
        self.h_out.copy_(self.batch.out, non_blocking=True)

    def __call__(self, host_coord, sync: bool = True):
        """One step on host coordinates.  With ``sync`` the device status is
        read as well: a candidate overflow doubles the capacity, captures the
        step again and repeats it (other statuses raise)."""
        self.h2d(host_coord)
        self.graph.replay()
        self.d2h()
        if sync:
            torch.cuda.current_stream(self.model.device).synchronize()
            st = self.batch.status()
            while st == L.GBDP_STATUS_CAND_OVERFLOW and self.batch.plan.grow_candidates():
                self._capture(1)
                self.graph.replay()
                self.d2h()
                torch.cuda.current_stream(self.model.device).synchronize()
                st = self.batch.status()
            if st != 0:
                raise L.GbdpError(f"fused step device status {st}: {L.GBDP_STATUS.get(st, '?')}")
        return self.h_energy, self.h_force, self.h_vir

    def status(self) -> int:
        return self.batch.status()


def build_model(cfg: mdl.SeAConfig, seed: int, stat_frames, device, dtype=torch.float32,
                compressed: bool = True):
    """Seeded parameters, davg/dstd from ``stat_frames`` (list of (coord,
    atype, box)) computed with the GPU env matrix, the minimum neighbour
    distance over them, and the tables."""
    params = mdl.init_params(cfg, seed)
    dev = torch.device(device)
    nn = cfg.nnei
    zeros = torch.zeros((cfg.ntypes, nn * 4), dtype=torch.float64, device=dev)
    ones = torch.ones((cfg.ntypes, nn * 4), dtype=torch.float64, device=dev)
    ems, ats = [], []
    mind = np.inf
    for c, t, b in stat_frames:
        plan = NeighborPlan([len(t)], np.asarray(b).reshape(1, 9), cfg.rcut, dev, torch.float64)
        r = env_mat_packed(plan, torch.tensor(c, dtype=torch.float64, device=dev),
                           torch.tensor(t, dtype=torch.int32, device=dev), zeros, ones,
                           cfg.rcut_smth, list(cfg.sel))
        ems.append(r.em.cpu().numpy())
        ats.append(np.asarray(t))
        d = torch.linalg.norm(r.rij.reshape(-1, 3), dim=1)
        d = d[r.nlist.reshape(-1) >= 0]
        if d.numel():
            mind = min(mind, float(d.min()))
    davg, dstd = mdl.stats_from_env(ems, ats, cfg)
    tables = infos = None
    if compressed:
        tables, infos = mdl.build_tables(params, davg, dstd, mind, cfg)
    model = SeAModel(cfg, params, davg, dstd, dev, dtype, tables, infos)
    model.params_np = params
    model.min_nbor_dist = mind
    model.tables_np = tables
    model.infos_np = infos
    return model
