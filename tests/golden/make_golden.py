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

Usage:  python tests/golden/make_golden.py [/path/to/reference]
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
REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"

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
    print("fixtures:", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
