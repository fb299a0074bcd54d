"""CPU composite of the whole se_e2_a energy / force / virial step — TEST
INFRASTRUCTURE ONLY (the parity reference for the GPU model and the timed
CPU baseline of bench.py).

It follows the reference's discrete-op sequence of the TF backend
(deepmd/tf/descriptor/se_a.py:652-765): ProdEnvMatA (internal periodic mode)
-> tabulated (or plain) embedding contracted with the env rows ->
descriptor -> fitting -> dE/d(env matrix) -> ProdForceSeA / ProdVirialSeA.
The env matrix, tabulation and force/virial steps call the oracle library
(restating source/lib/src/*.cc); the embedding and fitting nets, which the
reference runs as plain framework matmuls, are numpy (BLAS).
"""

from __future__ import annotations

import numpy as np

import oracle as O


def _tanh_layers_fwd(layers, x):
    """Embedding net (tanh, ResNet skip when width is kept or doubled);
    returns the output and the per-layer cache for the backward."""
    cache = []
    y = x
    for L in layers:
        t = np.tanh(y @ L["w"] + L["b"])
        out = t
        if L["skip"] == "same":
            out = out + y
        elif L["skip"] == "double":
            out = out + np.concatenate([y, y], -1)
        cache.append((y, t))
        y = out
    return y, cache


def _tanh_layers_bwd(layers, cache, g):
    for L, (y, t) in zip(reversed(layers), reversed(cache)):
        gz = g * (1 - t * t)
        gy = gz @ L["w"].T
        if L["skip"] == "same":
            gy = gy + g
        elif L["skip"] == "double":
            n = y.shape[-1]
            gy = gy + g[..., :n] + g[..., n:]
        g = gy
    return g


def fitting_energy_and_grad(fit, bias, D):
    """Per-atom energy of one type's fitting net and dE/dD (hidden layers
    tanh with idt and skip where present, then a linear output)."""
    h = D
    cache = []
    for L in fit["hidden"]:
        t = np.tanh(h @ L["w"] + L["b"])
        out = t * L["idt"] if L["idt"] is not None else t
        if L["skip"] == "same":
            out = out + h
        cache.append((h, t))
        h = out
    e = (h @ fit["final"]["w"] + fit["final"]["b"])[:, 0] + bias
    g = np.broadcast_to(fit["final"]["w"][:, 0], h.shape).copy()
    for L, (hin, t) in zip(reversed(fit["hidden"]), reversed(cache)):
        gt = g * L["idt"] if L["idt"] is not None else g
        gz = gt * (1 - t * t)
        gin = gz @ L["w"].T
        if L["skip"] == "same":
            gin = gin + g
        g = gin
    return e, g


def energy_force_virial(cfg, params, davg, dstd, coord, atype, box, tables=None,
                        table_infos=None, dtype=np.float64, cell_list=False):
    """One frame.  tables given -> compressed (tabulate ops); else plain
    embedding nets.  cell_list: O(N) cell-list candidate build (the
    reference's build_nlist) instead of the O(N^2) build_nlist_cpu; the
    results are identical.  Returns (energy, force [nloc,3], virial [9],
    atom_energy [nloc])."""
    sel = list(cfg.sel)
    nnei = cfg.nnei
    sec = cfg.sec
    M = cfg.neuron[-1]
    A = cfg.axis_neuron
    nloc = len(atype)
    em, emd, rij, nl = O.prod_env_mat_a_pbc(
        np.asarray(coord, dtype).reshape(-1), atype, np.asarray(box, dtype).reshape(-1),
        np.asarray(davg, dtype), np.asarray(dstd, dtype), cfg.rcut, cfg.rcut_smth, sel,
        cell_list=cell_list)
    em3 = em.reshape(nloc, nnei, 4)
    X = np.zeros((nloc, 4, M), dtype)
    saved = []
    for tj in range(cfg.ntypes):
        for ti in (range(cfg.ntypes) if not cfg.type_one_side else [None]):
            rows = np.arange(nloc) if ti is None else np.where(atype == ti)[0]
            if len(rows) == 0 or sel[tj] == 0:
                continue
            k = tj if cfg.type_one_side else tj * cfg.ntypes + ti
            rr = np.ascontiguousarray(em3[rows, sec[tj]:sec[tj + 1], :])
            ss = np.ascontiguousarray(rr[:, :, 0])
            if tables is not None:
                gr = O.tabulate_fusion_se_a(np.asarray(tables[k], dtype), np.asarray(table_infos[k], dtype),
                                            ss.reshape(-1, 1), rr, M)
                saved.append((rows, tj, k, rr, ss, None))
            else:
                gg, cache = _tanh_layers_fwd(params["emb"][k], ss[..., None])
                gr = np.einsum("njm,njk->nmk", rr, gg)
                saved.append((rows, tj, k, rr, ss, (gg, cache)))
            X[rows] += gr
    X /= nnei
    D = np.einsum("nmk,nma->nka", X, X[:, :, :A]).reshape(nloc, M * A)
    ae = np.zeros(nloc, dtype)
    dD = np.zeros_like(D)
    for t in range(cfg.ntypes):
        rows = np.where(atype == t)[0]
        if len(rows) == 0:
            continue
        e, g = fitting_energy_and_grad(params["fit"][t], params["bias_atom_e"][t], D[rows])
        ae[rows] = e
        dD[rows] = g
    G = dD.reshape(nloc, M, A)
    dX = np.einsum("nka,nma->nmk", G, X[:, :, :A])
    dX[:, :, :A] += np.einsum("nka,nmk->nma", G, X)
    dy = dX / nnei
    net = np.zeros((nloc, nnei, 4), dtype)
    for rows, tj, k, rr, ss, pl in saved:
        dyr = np.ascontiguousarray(dy[rows])
        if pl is None:
            gx, gm = O.tabulate_fusion_se_a_grad(np.asarray(tables[k], dtype), np.asarray(table_infos[k], dtype),
                                                 ss.reshape(-1, 1), rr, dyr)
            gm = gm.copy()
            gm[:, :, 0] += gx.reshape(gm.shape[:2])
        else:
            gg, cache = pl
            gm = np.einsum("nmk,njk->njm", dyr, gg)
            ggrad = np.einsum("nmk,njm->njk", dyr, rr)
            gs = _tanh_layers_bwd(params["emb"][k], cache, ggrad)
            gm[:, :, 0] += gs[..., 0]
        net[rows, sec[tj]:sec[tj + 1], :] += gm
    force = O.prod_force_a(net.reshape(-1), emd, nl, nloc, nloc, nnei).reshape(nloc, 3)
    vir, _ = O.prod_virial_a(net.reshape(-1), emd, rij, nl, nloc, nloc, nnei)
    return float(ae.astype(np.float64).sum()), force, vir, ae
