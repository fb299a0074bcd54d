"""se_e2_a energy model definition: configuration, seeded parameters,
descriptor statistics (davg / dstd) and the compression tables.

Architecture (deepmd/pt/model/descriptor/se_a.py, deepmd/pt/model/task/
fitting.py, deepmd/dpmodel/utils/network.py):
  * embedding nets 1 -> neuron[0] -> ... (tanh, ResNet skip when a layer keeps
    or doubles its width), one per neighbour type (type_one_side) or per
    (neighbour type, centre type) pair, indexed tj * ntypes + ti;
  * descriptor D = X^T X[:, :axis_neuron] with X = sum_j R_j^T G(s_j) / nnei;
  * fitting net per centre type: hidden layers (tanh; a time step idt and a
    skip only where the width is kept), then a linear layer to one energy.
Parameters are numpy float64; models cast them to their working dtype.
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class SeAConfig:
    ntypes: int = 2
    rcut: float = 6.0
    rcut_smth: float = 0.5
    sel: tuple = (46, 92)
    neuron: tuple = (25, 50, 100)
    axis_neuron: int = 16
    fitting: tuple = (240, 240, 240)
    type_one_side: bool = True
    resnet_dt: bool = True
    # compression (deepmd/utils/argcheck.py:2943-2965 defaults)
    extrapolate: float = 5.0
    stride0: float = 0.01
    stride1: float = 0.1

    @property
    def nnei(self) -> int:
        return int(sum(self.sel))

    @property
    def sec(self) -> list:
        return [0] + list(np.cumsum(self.sel))

    @property
    def n_emb(self) -> int:
        return self.ntypes if self.type_one_side else self.ntypes * self.ntypes

    @property
    def dim_descrpt(self) -> int:
        return self.neuron[-1] * self.axis_neuron


def _skip_kind(n_in: int, n_out: int) -> str:
    if n_in == n_out:
        return "same"
    if 2 * n_in == n_out:
        return "double"
    return "none"


def init_params(cfg: SeAConfig, seed: int) -> dict:
    """Seeded weights: W, b ~ N(0, 1/fan_in); idt ~ N(0.1, 0.001) where a
    skip connection exists (fitting); bias_atom_e = 0."""
    rng = np.random.default_rng(seed)
    emb = []
    for _ in range(cfg.n_emb):
        layers = []
        n_in = 1
        for n_out in cfg.neuron:
            sd = 1.0 / math.sqrt(n_in)
            layers.append({"w": rng.normal(0, sd, (n_in, n_out)), "b": rng.normal(0, sd, (n_out,)),
                           "skip": _skip_kind(n_in, n_out)})
            n_in = n_out
        emb.append(layers)
    fit = []
    for _ in range(cfg.ntypes):
        layers = []
        n_in = cfg.dim_descrpt
        for n_out in cfg.fitting:
            sd = 1.0 / math.sqrt(n_in)
            skip = _skip_kind(n_in, n_out)
            idt = rng.normal(0.1, 0.001, (n_out,)) if (cfg.resnet_dt and skip != "none") else None
            layers.append({"w": rng.normal(0, sd, (n_in, n_out)), "b": rng.normal(0, sd, (n_out,)),
                           "idt": idt, "skip": skip})
            n_in = n_out
        sd = 1.0 / math.sqrt(n_in)
        final = {"w": rng.normal(0, sd, (n_in, 1)), "b": rng.normal(0, sd, (1,))}
        fit.append({"hidden": layers, "final": final})
    return {"emb": emb, "fit": fit, "bias_atom_e": np.zeros(cfg.ntypes)}


# ----------------------------------------------------------- statistics --
def stats_from_env(em_list, atype_list, cfg: SeAConfig, protection: float = 1e-2):
    """davg / dstd from env matrices computed with avg 0 / std 1
    (deepmd/dpmodel/utils/env_mat_stat.py:137-340 and
    deepmd/utils/env_mat_stat.py:60-105): per centre type over every
    (atom, slot) entry, radial column r and the three angular columns a;
    davg = [avg_r, 0, 0, 0], dstd = [std_r, std_a, std_a, std_a] tiled over
    the nnei slots; std below ``protection`` is raised to it."""
    nn = cfg.nnei
    s = {t: np.zeros(6) for t in range(cfg.ntypes)}  # n_r, sum_r, sq_r, n_a, sum_a, sq_a
    for em, at in zip(em_list, atype_list):
        em = np.asarray(em, np.float64).reshape(-1, nn, 4)
        at = np.asarray(at).reshape(-1)
        for t in range(cfg.ntypes):
            dd = em[at == t]
            r = dd[..., 0]
            a = dd[..., 1:]
            s[t] += [r.size, r.sum(), (r * r).sum(), a.size, a.sum(), (a * a).sum()]
    davg = np.zeros((cfg.ntypes, nn * 4))
    dstd = np.ones((cfg.ntypes, nn * 4))

    def _std(n, sm, sq, default=1e-1):
        if n == 0:
            return default
        v = math.sqrt(max(sq / n - (sm / n) ** 2, 0.0))
        return protection if abs(v) < protection else v

    for t in range(cfg.ntypes):
        n_r, sum_r, sq_r, n_a, sum_a, sq_a = s[t]
        avg_r = sum_r / n_r if n_r else 0.0
        davg[t, 0::4] = avg_r
        dstd[t, 0::4] = _std(n_r, sum_r, sq_r)
        sa = _std(n_a, sum_a, sq_a)
        dstd[t, 1::4] = dstd[t, 2::4] = dstd[t, 3::4] = sa
    return davg, dstd


# -------------------------------------------------------------- tables --
def _spline5_switch(x: float, rmin: float, rmax: float) -> float:
    if x < rmin:
        return 1.0
    if x < rmax:
        u = (x - rmin) / (rmax - rmin)
        return u * u * u * (-6 * u * u + 15 * u - 10) + 1
    return 0.0


def embedding_value_and_derivs(layers, x: np.ndarray):
    """Value, first and second derivative wrt the scalar input of a tanh
    embedding net with ResNet skips, by the chain rule (the quantities of
    deepmd/utils/tabulate_math.py:353-470)."""
    x = x.reshape(-1, 1)
    y = x
    dy = np.ones_like(x)
    d2y = np.zeros_like(x)
    for L in layers:
        z = y @ L["w"] + L["b"]
        t = np.tanh(z)
        dt = 1 - t * t                    # tanh'
        dz = dy @ L["w"]
        d2z = d2y @ L["w"]
        val = t
        d1 = dt * dz
        d2 = -2 * t * dt * dz * dz + dt * d2z
        if L["skip"] == "same":
            val, d1, d2 = val + y, d1 + dy, d2 + d2y
        elif L["skip"] == "double":
            val = val + np.concatenate([y, y], 1)
            d1 = d1 + np.concatenate([dy, dy], 1)
            d2 = d2 + np.concatenate([d2y, d2y], 1)
        y, dy, d2y = val, d1, d2
    return y, dy, d2y


def build_tables(params: dict, davg: np.ndarray, dstd: np.ndarray, min_nbor_dist: float,
                 cfg: SeAConfig):
    """Fifth-order tables of every embedding net (DPTabulate.build for the
    "A" descriptor, deepmd/utils/tabulate.py:67-370, :468-486).

    Range, as the PyTorch descriptor's compression computes it: DescrptSeA
    keeps davg / dstd as [ntypes, nnei, 4] and DPTabulate.build
    (deepmd/utils/tabulate.py:90-95, :468-486) takes, per centre type, the
    four columns c of the first slot, lower_c = floor(-davg_c / dstd_c) and
    upper_c = ceil((sw(rmin) / rmin - davg_c) / dstd_c), and reduces them
    with min / max over c (so the angular columns, davg 0 and a smaller
    dstd, usually set the upper bound); a one-side net then takes the min /
    max over the centre types with a non-empty sel.  Rows of width stride0
    on [lower, upper) and stride1 on [upper, extrapolate * upper); each row
    holds, per output k, the six coefficients of the quintic Hermite
    interpolant matching value, first and second derivative at both ends.
    davg / dstd: [ntypes, nnei * 4] (or [ntypes, nnei, 4]).
    Returns (tables [n_emb] float64 [nspline, 6 M], infos [n_emb, 6])."""
    sw = _spline5_switch(min_nbor_dist, cfg.rcut_smth, cfg.rcut)
    a0 = np.asarray(davg, np.float64).reshape(cfg.ntypes, -1, 4)[:, 0, :]
    s0 = np.asarray(dstd, np.float64).reshape(cfg.ntypes, -1, 4)[:, 0, :]
    lo_t = np.floor(-a0 / s0).min(axis=1)
    up_t = np.ceil(((1.0 / min_nbor_dist) * sw - a0) / s0).max(axis=1)
    tables, infos = [], []
    M = cfg.neuron[-1]
    for k in range(cfg.n_emb):
        if cfg.type_one_side:
            valid = [t for t in range(cfg.ntypes) if cfg.sel[t] > 0]
            ll, uu = float(np.min(lo_t[valid])), float(np.max(up_t[valid]))
        else:
            ti = k % cfg.ntypes
            ll, uu = float(lo_t[ti]), float(up_t[ti])
        ext = cfg.extrapolate
        xx = np.arange(ll, uu, cfg.stride0)
        xx = np.append(xx, np.arange(uu, ext * uu, cfg.stride1))
        xx = np.append(xx, [ext * uu])
        nspline = int((uu - ll) / cfg.stride0 + (ext * uu - uu) / cfg.stride1)
        vv, dd, d2 = embedding_value_and_derivs(params["emb"][k], xx)
        tt = np.full((nspline, M), cfg.stride1)
        tt[: int((uu - ll) / cfg.stride0), :] = cfg.stride0
        hh = vv[1 : nspline + 1] - vv[:nspline]
        d0, d1 = dd[:nspline], dd[1 : nspline + 1]
        s0, s1 = d2[:nspline], d2[1 : nspline + 1]
        tab = np.zeros((nspline, 6 * M))
        tab[:, 0::6] = vv[:nspline]
        tab[:, 1::6] = d0
        tab[:, 2::6] = 0.5 * s0
        tab[:, 3::6] = (20 * hh - (8 * d1 + 12 * d0) * tt - (3 * s0 - s1) * tt * tt) / (2 * tt ** 3)
        tab[:, 4::6] = (-30 * hh + (14 * d1 + 16 * d0) * tt + (3 * s0 - 2 * s1) * tt * tt) / (2 * tt ** 4)
        tab[:, 5::6] = (12 * hh - 6 * (d1 + d0) * tt + (s1 - s0) * tt * tt) / (2 * tt ** 5)
        tables.append(tab)
        infos.append([ll, uu, uu * ext, cfg.stride0, cfg.stride1, -1.0])
    return tables, np.array(infos)
