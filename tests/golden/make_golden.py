"""Regenerate the golden fixtures in this directory.

Two sources, both read only here (the fixtures travel; the reference does not):

1. ``lib_tests.json`` / ``pt_tabulate.json``: the known-answer vectors that the
   reference's own tests hold for this path, read as TEXT from
   ``source/lib/tests/test_{env_mat_a,fmt_nlist,tabulate_se_a,prod_force_a,
   prod_virial_a,prod_force_grad_a,prod_virial_grad_a}.cc`` and
   ``source/tests/pt/test_tabulate_fusion_se_a.py``.
2. ``ref_water.npz``: outputs of the reference's own CPU library
   (``oracle/_ref/libref_cpu.so``, compiled from the reference sources by
   ``oracle/Makefile``) on seeded synthetic water frames.
3. ``ref_deeppot_sea.npz``: the reference's se_e2_a test model
   (``source/tests/infer/deeppot_sea.yaml``: descriptor statistics,
   embedding and fitting weights) and the energies, forces and virials its
   own inference test expects (``source/tests/infer/deeppot-testcase.yaml``),
   read with the package's YAML reader (``dpmd-public_gb300/serial.py``;
   PyYAML is not installed here) and stored in its flat format.
4. ``pt_format_nlist.npz``: the reference's own PyTorch neighbour-list
   formatting for ``forward_lower`` (``_format_nlist`` of
   ``deepmd/pt/model/model/make_model.py`` with the forced sort a compressed
   se_e2_a asks for, then ``nlist_distinguish_types`` of
   ``deepmd/pt/utils/nlist.py``), executed from its source on a seeded water
   frame whose candidate list is every extended atom within rcut + 2 A in a
   shuffled order, as an MD engine hands it over.

5. ``ref_tabulate.npz``: compression tables built by the reference's own
   ``DPTabulate`` (``deepmd/utils/tabulate_math.py`` on
   ``deepmd/utils/tabulate.py``, executed from their source with the numpy
   array namespace) for seeded se_e2_a embedding nets and statistics laid out
   as the PyTorch descriptor keeps them ([ntypes, nnei, 4]): a small net
   (widths 2-4-8, coarse strides) stored whole, and the bench-shaped net
   (25-50-100, strides 0.01 / 0.1, extrapolate 5) for both type_one_side
   settings stored as lower / upper / nspline, per-column sums and a sample
   of rows.

6. ``ref_descriptor_pt.npz``: the reference's own PyTorch descriptor
   (``DescrptSeA`` of ``deepmd/pt/model/descriptor/se_a.py``, compressed,
   FP64) run on CPU from a copy of the reference package with its own
   ``torch.ops.deepmd.tabulate_fusion_se_a`` compiled from
   ``source/op/pt/tabulate_multi_device.cc``: seeded weights and statistics,
   a seeded 192-atom water frame extended and listed by the reference's own
   ``extend_input_and_build_neighbor_list``; the descriptor, the gradient of
   a seeded linear function of it wrt the extended coordinates, and the
   ``tabulate_fusion_se_a`` calls the module made (inputs, outputs and
   input gradients for a seeded output gradient, first 24 atoms).  The
   package copy, the import stand-ins for packages this image lacks (yaml,
   dargs, h5py, wcmatch, mendeleev, lmdb, e3nn: never used on this path;
   array_api_compat: numpy / torch namespaces) and the compiled op live in
   a temporary directory only.

Usage:  python tests/golden/make_golden.py [/path/to/reference]
        (or DPMD_REFERENCE=/path/to/reference python tests/golden/make_golden.py)
"""

from __future__ import annotations

import ast
import importlib.util
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DPMD_REFERENCE", "")
if __name__ == "__main__" and not os.path.isdir(os.path.join(REF, "source")):
    sys.exit("make_golden.py: give the reference root as an argument or in DPMD_REFERENCE")

LIB_TESTS = [
    "test_env_mat_a.cc",
    "test_fmt_nlist.cc",
    "test_tabulate_se_a.cc",
    "test_prod_force_a.cc",
    "test_prod_virial_a.cc",
    "test_prod_force_grad_a.cc",
    "test_prod_virial_grad_a.cc",
]

_NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?")


def _numbers(body: str):
    vals = []
    for tok in _NUM.findall(body):
        vals.append(float(tok) if any(c in tok for c in ".eE") else int(tok))
    return vals


def parse_gtest_fixtures(path: str) -> dict:
    """Every ``class X : public ::testing::Test {`` body -> its vector
    literals, ``double box[] = {...}`` and scalar ``double/int name = v;``."""
    src = open(path).read()
    out = {}
    for m in re.finditer(r"class\s+(\w+)\s*:\s*public\s+::testing::Test\s*\{", src):
        name = m.group(1)
        depth, i = 1, m.end()
        while depth:
            depth += {"{": 1, "}": -1}.get(src[i], 0)
            i += 1
        body = src[m.end() : i]
        fx = {}
        for v in re.finditer(r"std::vector<[\w: ]+>\s+(\w+)\s*=\s*\{([^}]*)\};", body):
            fx[v.group(1)] = _numbers(v.group(2))
        for v in re.finditer(r"double\s+box\[\]\s*=\s*\{([^}]*)\};", body):
            fx["box"] = _numbers(v.group(1))
        for v in re.finditer(r"(?:const\s+)?(?:double|int)\s+(\w+)\s*=\s*([-+0-9.eE]+);", body):
            fx.setdefault(v.group(1), _numbers(v.group(2))[0])
        out[name] = fx
    return out


def parse_pt_tabulate(path: str) -> dict:
    """``self.<name> = torch.tensor([...]).reshape(...)`` assignments of the
    first TestCase in test_tabulate_fusion_se_a.py."""
    tree = ast.parse(open(path).read())
    out = {}
    for node in ast.walk(tree):
        if not (isinstance(node, ast.Assign) and len(node.targets) == 1):
            continue
        tgt = node.targets[0]
        if not (isinstance(tgt, ast.Attribute) and isinstance(tgt.value, ast.Name)):
            continue
        call = node.value
        shape = None
        if isinstance(call, ast.Call) and isinstance(call.func, ast.Attribute) and call.func.attr == "reshape":
            shape = [ast.literal_eval(a) for a in call.args]
            call = call.func.value
        if not (isinstance(call, ast.Call) and isinstance(call.func, ast.Attribute)
                and call.func.attr == "tensor" and call.args):
            continue
        try:
            vals = ast.literal_eval(call.args[0])
        except ValueError:
            continue
        if tgt.attr not in out:
            out[tgt.attr] = {"values": vals, "shape": shape}
    return out


def reference_water_fixture(path_out: str) -> None:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O  # noqa: E402

    if not O.have_ref():
        O.build(ref=True)
    spec = importlib.util.spec_from_file_location(
        "water", os.path.join(ROOT, "dpmd-public_gb300", "water.py"))
    W = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(W)
    sel = [46, 92]
    nnei = sum(sel)
    rng = np.random.default_rng(20261203)
    avg = np.zeros((2, nnei * 4))
    avg[:, 0::4] = rng.uniform(0.05, 0.15, (2, nnei))
    std = np.ones((2, nnei * 4))
    std[:, 0::4] = rng.uniform(0.1, 0.2, (2, nnei))
    std[:, 1::4] = std[:, 2::4] = std[:, 3::4] = rng.uniform(0.05, 0.1, (2, nnei))
    data = {"avg": avg, "std": std, "sel": np.array(sel), "rcut": 6.0, "rcut_smth": 0.5}
    frames = {"w192": (4, 12.42, 11), "w24": (2, 6.2, 12), "w1536": (8, 24.84, 13)}
    for tag, (n, L, seed) in frames.items():
        c, t, b = W.water_frame(n, L, seed)
        data[f"{tag}_coord"], data[f"{tag}_atype"], data[f"{tag}_box"] = c, t, b
        for dt, sfx in ((np.float64, "f64"), (np.float32, "f32")):
            em, emd, rij, nl, ec, et, emap = O.prod_env_mat_a_pbc(
                c.astype(dt), t, b.astype(dt), avg.astype(dt), std.astype(dt), 6.0, 0.5,
                sel, kind="ref", return_ext=True)
            data[f"{tag}_{sfx}_nlist"] = nl.astype(np.int16)
            data[f"{tag}_{sfx}_nall"] = len(et)
            data[f"{tag}_{sfx}_mapping"] = emap.astype(np.int16)
            keep = 24 * nnei  # first 24 centres only, to keep the file small
            data[f"{tag}_{sfx}_em"] = em[: keep * 4]
            data[f"{tag}_{sfx}_em_deriv"] = emd[: keep * 12]
            data[f"{tag}_{sfx}_rij"] = rij[: keep * 3]
            data[f"{tag}_{sfx}_em_sum"] = np.array([em.sum(), np.abs(emd).sum(), np.abs(rij).sum()])
    np.savez_compressed(path_out, **data)


def reference_model_fixture(path_out: str) -> None:
    sys.path.insert(0, ROOT)
    from __graft_entry__ import load_package  # noqa: E402

    load_package()
    import dpmd_public_gb300.serial as S  # noqa: E402

    with open(os.path.join(REF, "source/tests/infer/deeppot_sea.yaml")) as fh:
        cfg, params, davg, dstd, type_map = S.se_a_from_dict(S.parse_block_yaml(fh.read()))
    data = S.flatten(cfg, params, davg, dstd, type_map)
    case = open(os.path.join(REF, "source/tests/infer/deeppot-testcase.yaml")).read()
    blocks = re.split(r"\n\s*- coord:", case.split("results:", 1)[1])[1:]
    for n, blk in enumerate(blocks):
        blk = "coord:" + blk
        for key in ("coord", "atype", "box", "atomic_energy", "force", "atomic_virial"):
            mm = re.search(rf"\b{key}:\s*(null|\[[^\]]*\])", blk, re.S)
            if mm and mm.group(1) != "null":
                data[f"case{n}_{key}"] = np.array([float(x) for x in _NUM.findall(mm.group(1))])
    data["ncases"] = len(blocks)
    np.savez_compressed(path_out, **data)


def _reference_functions(names: dict) -> dict:
    """Compile the named functions from the reference sources (file -> names)
    into one namespace with torch: the reference's own code, run here."""
    import torch

    ns = {"torch": torch}
    for rel, fn_names in names.items():
        tree = ast.parse(open(os.path.join(REF, rel)).read())
        for node in ast.walk(tree):
            if isinstance(node, ast.FunctionDef) and node.name in fn_names:
                node.decorator_list = []
                mod = ast.Module(body=[node], type_ignores=[])
                exec(compile(mod, rel, "exec"), ns)
    return ns


def reference_format_nlist_fixture(path_out: str) -> None:
    import torch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O  # noqa: E402

    ns = _reference_functions({
        "deepmd/pt/model/model/make_model.py": {"_format_nlist"},
        "deepmd/pt/utils/nlist.py": {"nlist_distinguish_types"},
    })
    spec = importlib.util.spec_from_file_location(
        "water", os.path.join(ROOT, "dpmd-public_gb300", "water.py"))
    W = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(W)
    sel, rcut, skin = [46, 92], 6.0, 2.0
    c, t, b = W.water_frame(4, 12.42, 21)
    nloc = len(t)
    ext, etype, emap = O.copy_coord(c, t, b, rcut + skin)
    ext = ext.reshape(-1, 3)
    rng = np.random.default_rng(5438)
    cand = []
    for i in range(nloc):
        d = np.linalg.norm(ext - ext[i], axis=1)
        js = np.nonzero((d <= rcut + skin) & (np.arange(len(ext)) != i))[0]
        cand.append(rng.permutation(js))
    nnei_in = max(len(x) for x in cand) + 3
    nl_in = -np.ones((nloc, nnei_in), np.int64)
    for i, js in enumerate(cand):
        nl_in[i, : len(js)] = js
    data = {"ext_coord": ext, "ext_type": etype.astype(np.int32), "nlist_in": nl_in.astype(np.int32),
            "mapping": emap.astype(np.int32), "coord": c, "atype": t, "box": b,
            "nloc": nloc, "sel": np.array(sel), "rcut": rcut}

    class _Desc:
        def get_rcut(self):
            return rcut

    for dt, sfx in ((torch.float64, "f64"), (torch.float32, "f32")):
        ec = torch.tensor(ext[None], dtype=dt)
        nl = ns["_format_nlist"](_Desc(), ec, torch.tensor(nl_in[None]), sum(sel),
                                 extra_nlist_sort=True)
        nl = ns["nlist_distinguish_types"](nl, torch.tensor(etype[None], dtype=torch.int64), sel)
        data[f"{sfx}_nlist"] = nl[0].numpy().astype(np.int32)
    np.savez_compressed(path_out, **data)


def _reference_tabulate_module():
    """deepmd.utils.tabulate and deepmd.utils.tabulate_math executed from the
    reference sources, with the numpy array namespace standing in for
    array_api_compat and the two dpmodel helpers they import."""
    import types

    saved = {k: sys.modules.get(k) for k in (
        "array_api_compat", "deepmd", "deepmd.dpmodel", "deepmd.dpmodel.common",
        "deepmd.dpmodel.utils", "deepmd.dpmodel.utils.network", "deepmd.utils",
        "deepmd.utils.tabulate", "deepmd.utils.tabulate_math")}
    aac = types.ModuleType("array_api_compat")
    aac.array_namespace = lambda *xs: np
    aac.device = lambda x: "cpu"
    sys.modules["array_api_compat"] = aac
    for name in ("deepmd", "deepmd.dpmodel", "deepmd.dpmodel.utils", "deepmd.utils"):
        m = types.ModuleType(name)
        m.__path__ = []
        sys.modules[name] = m
    common = types.ModuleType("deepmd.dpmodel.common")
    common.to_numpy_array = lambda x: None if x is None else np.asarray(x)
    sys.modules["deepmd.dpmodel.common"] = common
    net = types.ModuleType("deepmd.dpmodel.utils.network")
    net.get_activation_fn = lambda name: {"tanh": np.tanh}[name]
    sys.modules["deepmd.dpmodel.utils.network"] = net
    mods = {}
    for name, rel in (("deepmd.utils.tabulate", "deepmd/utils/tabulate.py"),
                      ("deepmd.utils.tabulate_math", "deepmd/utils/tabulate_math.py")):
        spec = importlib.util.spec_from_file_location(name, os.path.join(REF, rel))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
        mods[name] = mod
    tm = mods["deepmd.utils.tabulate_math"]
    for k, v in saved.items():
        if v is None:
            sys.modules.pop(k, None)
        else:
            sys.modules[k] = v
    return tm


def reference_tabulate_fixture(path_out: str) -> None:
    sys.path.insert(0, ROOT)
    from __graft_entry__ import load_package  # noqa: E402

    load_package()
    import dataclasses

    import dpmd_public_gb300.model as mdl  # noqa: E402

    tm = _reference_tabulate_module()

    class _SeA:
        """The descriptor interface DPTabulate reads (get_sel, get_rcut,
        get_rcut_smth, get_ntypes, serialize), over seeded parameters."""

        def __init__(self, cfg, params, davg, dstd):
            self.cfg = cfg
            nets = [{"layers": [{"@variables": {"w": np.asarray(l["w"]), "b": np.asarray(l["b"])}}
                                for l in net]} for net in params["emb"]]
            self.ser = {"type": "se_e2_a",
                        "@variables": {"davg": davg.reshape(cfg.ntypes, cfg.nnei, 4),
                                       "dstd": dstd.reshape(cfg.ntypes, cfg.nnei, 4)},
                        "embeddings": {"networks": nets}}

        def get_sel(self):
            return list(self.cfg.sel)

        def get_rcut(self):
            return self.cfg.rcut

        def get_rcut_smth(self):
            return self.cfg.rcut_smth

        def get_ntypes(self):
            return self.cfg.ntypes

        def serialize(self):
            return self.ser

    def stats(cfg, seed):
        rng = np.random.default_rng(seed)
        nn = cfg.nnei
        davg = np.zeros((cfg.ntypes, nn * 4))
        davg[:, 0::4] = rng.uniform(0.03, 0.08, (cfg.ntypes, 1))
        dstd = np.ones((cfg.ntypes, nn * 4))
        dstd[:, 0::4] = rng.uniform(0.11, 0.15, (cfg.ntypes, 1))
        dstd[:, 1::4] = dstd[:, 2::4] = dstd[:, 3::4] = rng.uniform(0.07, 0.09, (cfg.ntypes, 1))
        return davg, dstd

    data = {}
    cases = {
        "small": (dataclasses.replace(mdl.SeAConfig(), neuron=(2, 4, 8), stride0=0.1, stride1=1.0),
                  0.9, 101),
        "bench_one_side": (mdl.SeAConfig(), 0.78, 20261203),
        "bench_pair": (dataclasses.replace(mdl.SeAConfig(), type_one_side=False), 0.78, 20261203),
    }
    rng = np.random.default_rng(77)
    for tag, (cfg, rmin, seed) in cases.items():
        params = mdl.init_params(cfg, seed)
        davg, dstd = stats(cfg, seed + 1)
        tab = tm.DPTabulate(_SeA(cfg, params, davg, dstd), list(cfg.neuron),
                            type_one_side=cfg.type_one_side)
        lower, upper = tab.build(rmin, cfg.extrapolate, cfg.stride0, cfg.stride1)
        data[f"{tag}_davg"], data[f"{tag}_dstd"], data[f"{tag}_rmin"] = davg, dstd, rmin
        data[f"{tag}_seed"] = seed
        names = list(tab.data)
        data[f"{tag}_nets"] = np.array(names)
        for k, name in enumerate(names):
            t = np.asarray(tab.data[name], np.float64)
            data[f"{tag}_{k}_lower"] = float(lower[name])
            data[f"{tag}_{k}_upper"] = float(upper[name])
            data[f"{tag}_{k}_nspline"] = t.shape[0]
            data[f"{tag}_{k}_colsum"] = np.abs(t).reshape(t.shape[0], -1, 6).sum(axis=(0, 1))
            if tag == "small":
                data[f"{tag}_{k}_table"] = t
            else:
                rows = np.unique(np.concatenate([[0, t.shape[0] - 1],
                                                 rng.integers(0, t.shape[0], 10)]))
                data[f"{tag}_{k}_rows"] = rows
                data[f"{tag}_{k}_sample"] = t[rows]
    np.savez_compressed(path_out, **data)


def _reference_pt_package(tmp: str):
    """A copy of the reference Python package in ``tmp`` with the metadata
    files its build would write, its PyTorch op library compiled from the
    reference sources, and import stand-ins for the packages this image
    lacks.  Returns the imported descriptor module and the nlist module."""
    import shutil
    import subprocess
    import types

    import torch
    import torch.utils.cpp_extension as ce

    shutil.copytree(os.path.join(REF, "deepmd"), os.path.join(tmp, "deepmd"))
    with open(os.path.join(tmp, "deepmd", "__about__.py"), "w") as fh:
        fh.write('__version__ = "0.0.0"\n')
    os.makedirs(os.path.join(tmp, "deepmd", "lib"), exist_ok=True)
    open(os.path.join(tmp, "deepmd", "lib", "__init__.py"), "w").close()
    tmpl = open(os.path.join(REF, "source", "config", "run_config.ini")).read()
    with open(os.path.join(tmp, "deepmd", "lib", "run_config.ini"), "w") as fh:
        fh.write(re.sub(r"@[^@]*@", "", tmpl))
    srcs = [os.path.join(REF, "source", "op", "pt", f)
            for f in ("tabulate_multi_device.cc", "print_summary.cc")]
    srcs += [os.path.join(REF, "source", "lib", "src", f) for f in ("tabulate.cc", "errors.cc")
             if os.path.exists(os.path.join(REF, "source", "lib", "src", f))]
    lib = ce.library_paths()[0]
    cmd = (["g++", "-O2", "-shared", "-fPIC", "-std=c++17",
            f"-D_GLIBCXX_USE_CXX11_ABI={int(torch._C._GLIBCXX_USE_CXX11_ABI)}",
            "-I" + os.path.join(REF, "source", "lib", "include")]
           + [f"-I{p}" for p in ce.include_paths()] + srcs
           + [f"-L{lib}", f"-Wl,-rpath,{lib}", "-ltorch", "-ltorch_cpu", "-lc10", "-o",
              os.path.join(tmp, "deepmd", "lib", "libdeepmd_op_pt.so")])
    subprocess.run(cmd, check=True)

    class _Absent(types.ModuleType):
        def __getattr__(self, name):
            if name.startswith("__"):
                raise AttributeError(name)
            return type(name, (), {"__init__": lambda s_, *a, **k: None,
                                   "__call__": lambda s_, *a, **k: None})

    for m in ("yaml", "dargs", "h5py", "wcmatch", "wcmatch.glob", "mendeleev", "lmdb", "e3nn",
              "e3nn.o3"):
        sys.modules.setdefault(m, _Absent(m))

    class _TorchNS:
        def __getattr__(self, n):
            return getattr(torch, n)

        def astype(self, x, dtype, copy=True):
            return x.to(dtype)

        def asarray(self, x, dtype=None, device=None, copy=None):
            return torch.as_tensor(x, dtype=dtype, device=device)

        def concat(self, xs, axis=0):
            return torch.cat(xs, dim=axis)

        def permute_dims(self, x, axes):
            return x.permute(*axes)

        def expand_dims(self, x, axis):
            return x.unsqueeze(axis)

        def sum(self, x, axis=None, keepdims=False):
            return x.sum() if axis is None else x.sum(dim=axis, keepdim=keepdims)

        def reshape(self, x, shape):
            return x.reshape(shape)

    tns = _TorchNS()
    aac = types.ModuleType("array_api_compat")
    aac.array_namespace = lambda *xs: tns if any(isinstance(x, torch.Tensor) for x in xs) else np
    aac.device = lambda x: getattr(x, "device", "cpu")
    aac.is_torch_array = lambda x: isinstance(x, torch.Tensor)
    aac.is_numpy_array = lambda x: isinstance(x, np.ndarray)
    aac.is_array_api_obj = lambda x: isinstance(x, (np.ndarray, torch.Tensor))
    aac.to_device = lambda x, d: x
    aac.size = lambda x: x.size if isinstance(x, np.ndarray) else x.numel()
    sys.modules["array_api_compat"] = aac
    sys.path.insert(0, tmp)
    import deepmd.pt.model.descriptor.se_a as S  # noqa: E402
    import deepmd.pt.utils.nlist as NL  # noqa: E402

    return S, NL


def reference_descriptor_fixture(path_out: str) -> None:
    import tempfile

    import torch

    sys.path.insert(0, ROOT)
    from __graft_entry__ import load_package  # noqa: E402

    load_package()
    import dpmd_public_gb300.model as mdl  # noqa: E402
    import dpmd_public_gb300.water as W  # noqa: E402

    torch.set_default_dtype(torch.float64)
    with tempfile.TemporaryDirectory() as tmp:
        S, NL = _reference_pt_package(tmp)
        cfg = mdl.SeAConfig()
        seed = 2026
        params = mdl.init_params(cfg, seed)
        rng = np.random.default_rng(seed + 1)
        nn = cfg.nnei
        davg = np.zeros((cfg.ntypes, nn, 4))
        davg[:, :, 0] = rng.uniform(0.03, 0.08, (cfg.ntypes, 1))
        dstd = np.ones((cfg.ntypes, nn, 4))
        dstd[:, :, 0] = rng.uniform(0.11, 0.15, (cfg.ntypes, 1))
        dstd[:, :, 1:] = rng.uniform(0.07, 0.09, (cfg.ntypes, 1, 1))
        rmin = 0.78
        d = S.DescrptSeA(rcut=cfg.rcut, rcut_smth=cfg.rcut_smth, sel=list(cfg.sel),
                         neuron=list(cfg.neuron), axis_neuron=cfg.axis_neuron,
                         type_one_side=True, precision="float64", resnet_dt=False)
        ser = d.serialize()
        for k, net in enumerate(ser["embeddings"]["networks"]):
            for l, layer in enumerate(net["layers"]):
                layer["@variables"]["w"] = np.asarray(params["emb"][k][l]["w"], np.float64)
                layer["@variables"]["b"] = np.asarray(params["emb"][k][l]["b"], np.float64)
        ser["@variables"]["davg"] = davg
        ser["@variables"]["dstd"] = dstd
        d = S.DescrptSeA.deserialize(ser)
        d.enable_compression(rmin, 5, 0.01, 0.1)
        calls = []
        real = torch.ops.deepmd.tabulate_fusion_se_a

        def record(table, info, em_x, em, last):
            out = real(table, info, em_x, em, last)
            calls.append((info.detach().clone(), em_x.detach().clone(), em.detach().clone(),
                          out[0].detach().clone(), int(last)))
            return out

        torch.ops.deepmd.tabulate_fusion_se_a = record
        c, t, b = W.water_frame(4, 12.42, 2027)
        coord = torch.tensor(c[None])
        atype = torch.tensor(t[None], dtype=torch.int64)
        box = torch.tensor(b[None])
        ext, etype, mapping, nlist = NL.extend_input_and_build_neighbor_list(
            coord, atype, cfg.rcut, list(cfg.sel), mixed_types=False, box=box)
        ext = ext.detach().clone().requires_grad_(True)
        desc = d(ext.reshape(1, -1), etype, nlist, mapping)[0]
        wts = torch.tensor(np.random.default_rng(seed + 2).normal(0, 1, desc.shape))
        (grad,) = torch.autograd.grad((desc * wts).sum(), ext)
        torch.ops.deepmd.tabulate_fusion_se_a = real
        keep = 24
        data = {"seed": seed, "davg": davg.reshape(cfg.ntypes, -1), "dstd": dstd.reshape(cfg.ntypes, -1),
                "rmin": rmin, "coord": c, "atype": t, "box": b,
                "ext_coord": ext.detach().numpy()[0], "ext_atype": etype.numpy()[0].astype(np.int32),
                "mapping": mapping.numpy()[0].astype(np.int32),
                "nlist": nlist.numpy()[0].astype(np.int32),
                "desc_head": desc.detach().numpy()[0, :keep],
                "desc_norm": np.linalg.norm(desc.detach().numpy()[0], axis=1),
                "grad_ext": grad.numpy()[0],
                "ncalls": len(calls)}
        for q, (info, em_x, em, out, last) in enumerate(calls):
            nsel = em.shape[1]
            data[f"call{q}_info"] = info.numpy()
            data[f"call{q}_last"] = last
            data[f"call{q}_em"] = em.numpy()[:keep]
            data[f"call{q}_em_x"] = em_x.numpy()[: keep * nsel]
            data[f"call{q}_out"] = out.numpy()[:keep]
            dy = torch.tensor(np.random.default_rng(seed + 10 + q).normal(0, 1, (keep, 4, last)))
            ex = em_x[: keep * nsel].clone().requires_grad_(True)
            ee = em[:keep].clone().requires_grad_(True)
            tab = d.sea.compress_data[q].detach()
            data[f"call{q}_table_rows"] = tab.shape[0]
            data[f"call{q}_table_abs_sum"] = float(tab.abs().sum())
            o = real(tab, info, ex, ee, last)[0]
            gx, gm = torch.autograd.grad(o, (ex, ee), dy)
            data[f"call{q}_dy"] = dy.numpy()
            data[f"call{q}_gx"] = gx.numpy()
            data[f"call{q}_gm"] = gm.numpy()
    np.savez_compressed(path_out, **data)


def main() -> None:
    lib = {}
    for f in LIB_TESTS:
        for k, v in parse_gtest_fixtures(os.path.join(REF, "source/lib/tests", f)).items():
            lib[k] = v
    with open(os.path.join(HERE, "lib_tests.json"), "w") as fh:
        json.dump(lib, fh, separators=(",", ":"))
    pt = parse_pt_tabulate(os.path.join(REF, "source/tests/pt/test_tabulate_fusion_se_a.py"))
    with open(os.path.join(HERE, "pt_tabulate.json"), "w") as fh:
        json.dump(pt, fh, separators=(",", ":"))
    reference_water_fixture(os.path.join(HERE, "ref_water.npz"))
    reference_format_nlist_fixture(os.path.join(HERE, "pt_format_nlist.npz"))
    reference_model_fixture(os.path.join(HERE, "ref_deeppot_sea.npz"))
    reference_tabulate_fixture(os.path.join(HERE, "ref_tabulate.npz"))
    reference_descriptor_fixture(os.path.join(HERE, "ref_descriptor_pt.npz"))
    print("fixtures:", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
