"""Load a trained se_e2_a energy model from the reference's serialized form.

The reference serializes models as nested dicts (``Model.serialize`` ->
``deepmd/dpmodel/model/make_model.py``, ``DescrptSeA.serialize``
``deepmd/dpmodel/descriptor/se_e2_a.py``, ``EnergyFittingNet.serialize``
``deepmd/dpmodel/fitting/general_fitting.py``) and writes them as YAML
(``deepmd/dpmodel/utils/serialization.py``), e.g. its inference test model
``source/tests/infer/deeppot_sea.yaml``.  This module reads the block-style
YAML subset those files use (PyYAML is not required) and maps the se_e2_a
descriptor and energy fitting onto ``model.SeAConfig`` and the parameter
layout ``se_a.SeAModel`` takes; ``flatten`` / ``unflatten`` store the same in
a flat ``.npz``.
"""

from __future__ import annotations

import json
import re

import numpy as np

from . import model as mdl


# ------------------------------------------------------------------ YAML --
def _scalar(s: str):
    s = s.strip()
    if s in ("null", "~", ""):
        return None
    if s in ("true", "false"):
        return s == "true"
    if s[:1] in "\"'" and s[-1:] == s[:1]:
        return s[1:-1]
    if s[:1] in "[{":
        return json.loads(s.replace("True", "true").replace("False", "false"))
    for conv in (int, float):
        try:
            return conv(s)
        except ValueError:
            pass
    return s


def parse_block_yaml(text: str):
    """The block-style YAML PyYAML writes for serialized models: nested
    mappings, sequences (including the ``- - -`` form of nested lists) and
    plain, quoted or one-line flow scalars.  Raises ValueError on anything
    else."""
    lines = []
    for raw in text.splitlines():
        s = raw.rstrip()
        if not s.strip() or s.lstrip().startswith("#"):
            continue
        ind = len(s) - len(s.lstrip())
        c = s.lstrip()
        while c == "-" or c.startswith("- "):
            lines.append((ind, "-"))
            c = c[2:].lstrip() if c != "-" else ""
            ind += 2
        if c:
            lines.append((ind, c))
    if not lines:
        return None
    pos = 0

    def node(ind):
        nonlocal pos
        if lines[pos][1] == "-":
            out = []
            while pos < len(lines) and lines[pos][0] == ind and lines[pos][1] == "-":
                pos += 1
                out.append(node(lines[pos][0])
                           if pos < len(lines) and lines[pos][0] > ind else None)
            return out
        if ":" not in lines[pos][1] or lines[pos][1][:1] in "[{":
            pos += 1
            return _scalar(lines[pos - 1][1])
        out = {}
        while pos < len(lines) and lines[pos][0] == ind and lines[pos][1] != "-":
            m = re.match(r'^("[^"]*"|\'[^\']*\'|[^:]+):(\s+(.*))?$', lines[pos][1])
            if not m:
                raise ValueError(f"unsupported YAML line: {lines[pos][1]!r}")
            key, rest = _scalar(m.group(1)), m.group(3)
            pos += 1
            if rest:
                out[key] = _scalar(rest)
            elif pos < len(lines) and (lines[pos][0] > ind or
                                       (lines[pos][0] == ind and lines[pos][1] == "-")):
                out[key] = node(lines[pos][0])
            else:
                out[key] = None
        return out

    return node(lines[0][0])


# ---------------------------------------------------------------- se_e2_a --
def _arr(v):
    return np.asarray(v["value"] if isinstance(v, dict) else v, np.float64)


def se_a_from_dict(d: dict):
    """(SeAConfig, params, davg [ntypes, nnei*4], dstd, type_map) from a
    serialized energy model whose descriptor is se_e2_a."""
    m = d.get("model", d)
    de, fi = m["descriptor"], m["fitting"]
    if de.get("type") != "se_e2_a":
        raise ValueError(f"descriptor {de.get('type')!r} is not se_e2_a")
    if fi.get("type") != "ener":
        raise ValueError(f"fitting {fi.get('type')!r} is not an energy fitting")
    if de.get("exclude_types") or m.get("atom_exclude_types") or m.get("pair_exclude_types"):
        raise ValueError("type exclusions are not supported")
    if fi.get("numb_fparam") or fi.get("numb_aparam"):
        raise ValueError("frame / atomic parameters are not supported")
    if de.get("env_protection", 0.0):
        raise ValueError("env_protection != 0 is not supported")
    sel = [int(x) for x in de["sel"]]
    cfg = mdl.SeAConfig(ntypes=len(sel), rcut=float(de["rcut"]), rcut_smth=float(de["rcut_smth"]),
                        sel=tuple(sel), neuron=tuple(int(x) for x in de["neuron"]),
                        axis_neuron=int(de["axis_neuron"]),
                        fitting=tuple(int(x) for x in fi["neuron"]),
                        type_one_side=bool(de["type_one_side"]), resnet_dt=bool(fi["resnet_dt"]))
    emb = []
    for net in de["embeddings"]["networks"]:
        layers, n_in = [], 1
        for layer in net["layers"]:
            w, b = _arr(layer["@variables"]["w"]), _arr(layer["@variables"]["b"])
            skip = mdl._skip_kind(n_in, w.shape[1]) if layer.get("resnet", True) else "none"
            layers.append({"w": w, "b": b, "skip": skip})
            n_in = w.shape[1]
        emb.append(layers)
    fit = []
    for net in fi["nets"]["networks"]:
        *hidden_l, final_l = net["layers"]
        hidden, n_in = [], cfg.dim_descrpt
        for layer in hidden_l:
            v = layer["@variables"]
            w, b = _arr(v["w"]), _arr(v["b"])
            skip = mdl._skip_kind(n_in, w.shape[1]) if layer.get("resnet", True) else "none"
            idt = _arr(v["idt"]) if v.get("idt") is not None else None
            hidden.append({"w": w, "b": b, "idt": idt, "skip": skip})
            n_in = w.shape[1]
        fv = final_l["@variables"]
        fit.append({"hidden": hidden, "final": {"w": _arr(fv["w"]), "b": _arr(fv["b"])}})
    nnei4 = cfg.nnei * 4
    davg = _arr(de["@variables"]["davg"]).reshape(cfg.ntypes, nnei4)
    dstd = _arr(de["@variables"]["dstd"]).reshape(cfg.ntypes, nnei4)
    bias = _arr(fi["@variables"]["bias_atom_e"]).reshape(-1)
    if "@variables" in m and "out_bias" in m["@variables"]:
        # the model's output statistics: e * out_std + out_bias per type
        ob = _arr(m["@variables"]["out_bias"]).reshape(-1)
        os_ = _arr(m["@variables"]["out_std"]).reshape(-1)
        if np.any(os_ != 1.0):
            raise ValueError("out_std != 1 is not supported")
        bias = bias + ob
    params = {"emb": emb, "fit": fit, "bias_atom_e": bias}
    return cfg, params, davg, dstd, list(de.get("type_map") or [])


def load_se_a(path: str):
    """(SeAConfig, params, davg, dstd, type_map) from a serialized model
    (``.yaml`` as the reference writes it, or ``.npz`` from ``flatten``)."""
    if path.endswith(".npz"):
        return unflatten(dict(np.load(path)))
    with open(path) as fh:
        return se_a_from_dict(parse_block_yaml(fh.read()))


def flatten(cfg, params, davg, dstd, type_map=()) -> dict:
    """Flat arrays for ``np.savez`` (the inverse of ``unflatten``)."""
    out = {"sel": np.array(cfg.sel), "neuron": np.array(cfg.neuron),
           "axis_neuron": cfg.axis_neuron, "rcut": cfg.rcut, "rcut_smth": cfg.rcut_smth,
           "fit_neuron": np.array(cfg.fitting), "type_one_side": int(cfg.type_one_side),
           "resnet_dt": int(cfg.resnet_dt), "davg": davg, "dstd": dstd,
           "bias_atom_e": np.asarray(params["bias_atom_e"]), "type_map": np.array(list(type_map))}
    for k, net in enumerate(params["emb"]):
        for l, layer in enumerate(net):
            out[f"emb{k}_l{l}_w"], out[f"emb{k}_l{l}_b"] = layer["w"], layer["b"]
    for t, net in enumerate(params["fit"]):
        for l, layer in enumerate(net["hidden"]):
            out[f"fit{t}_l{l}_w"], out[f"fit{t}_l{l}_b"] = layer["w"], layer["b"]
            if layer["idt"] is not None:
                out[f"fit{t}_l{l}_idt"] = layer["idt"]
        out[f"fit{t}_out_w"], out[f"fit{t}_out_b"] = net["final"]["w"], net["final"]["b"]
    return out


def unflatten(d: dict):
    sel = tuple(int(x) for x in d["sel"])
    cfg = mdl.SeAConfig(ntypes=len(sel), rcut=float(d["rcut"]), rcut_smth=float(d["rcut_smth"]),
                        sel=sel, neuron=tuple(int(x) for x in d["neuron"]),
                        axis_neuron=int(d["axis_neuron"]),
                        fitting=tuple(int(x) for x in d["fit_neuron"]),
                        type_one_side=bool(int(d["type_one_side"])),
                        resnet_dt=bool(int(d["resnet_dt"])))
    emb = []
    for k in range(cfg.n_emb):
        layers, n_in = [], 1
        for l in range(len(cfg.neuron)):
            w = np.asarray(d[f"emb{k}_l{l}_w"])
            layers.append({"w": w, "b": np.asarray(d[f"emb{k}_l{l}_b"]),
                           "skip": mdl._skip_kind(n_in, w.shape[1])})
            n_in = w.shape[1]
        emb.append(layers)
    fit = []
    for t in range(cfg.ntypes):
        hidden, n_in = [], cfg.dim_descrpt
        for l in range(len(cfg.fitting)):
            w = np.asarray(d[f"fit{t}_l{l}_w"])
            idt = d.get(f"fit{t}_l{l}_idt")
            hidden.append({"w": w, "b": np.asarray(d[f"fit{t}_l{l}_b"]),
                           "idt": None if idt is None else np.asarray(idt),
                           "skip": mdl._skip_kind(n_in, w.shape[1])})
            n_in = w.shape[1]
        fit.append({"hidden": hidden, "final": {"w": np.asarray(d[f"fit{t}_out_w"]),
                                                "b": np.asarray(d[f"fit{t}_out_b"])}})
    params = {"emb": emb, "fit": fit, "bias_atom_e": np.asarray(d["bias_atom_e"], np.float64)}
    tm = [str(x) for x in d.get("type_map", [])]
    return cfg, params, np.asarray(d["davg"]), np.asarray(d["dstd"]), tm
