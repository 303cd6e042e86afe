"""Regenerate the golden fixtures in this folder from the reference checkout.

Reads, as data:
  * the known-answer tests of tests/test_implicit_networks.cpp (TEST_CASE / SECTION blocks:
    the function file, the tet mesh, and the REQUIREd patch count, chain count, corner count and
    patch_function_label list);
  * the function lists examples/tests/*.json and the tet mesh examples/tests/mesh.json.
  * the CSG known answers of the same file (the lambda over cell labels, written here as a CSG tree;
    the REQUIREd patch, chain and corner counts and the patch_sign_label list).
Writes kat.json, csg_kat.json, functions/*.json and mesh_8sphere.npz next to this script.

Usage: python tests/golden/make_golden.py REFERENCE_ROOT
Nothing else reads the reference checkout; the tests only read the files written here.
"""
import json
import os
import re
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_kats(src: str):
    lines = src.splitlines()
    cases = []
    case_name = None
    cur = None
    for ln, line in enumerate(lines, 1):
        m = re.search(r'TEST_CASE\("([^"]+)"', line)
        if m:
            case_name = m.group(1)
            continue
        m = re.search(r'SECTION\("([^"]+)"\)', line)
        if m:
            cur = {"test_case": case_name, "section": m.group(1), "line": ln, "mesh": "grid101"}
            cases.append(cur)
            continue
        if cur is None:
            continue
        m = re.search(r'load_functions\(std::string\(TEST_FILE\) \+ "/([^"]+)\.json"', line)
        if m:
            cur["functions"] = m.group(1)
        if "load_tet_mesh" in line and "mesh.json" in line:
            cur["mesh"] = "mesh"
        m = re.search(r"REQUIRE\(patches\.size\(\) == (\d+)\)", line)
        if m:
            cur["patches"] = int(m.group(1))
        m = re.search(r"REQUIRE\(chains\.size\(\) == (\d+)\)", line)
        if m:
            cur["chains"] = int(m.group(1))
        m = re.search(r"REQUIRE\(corners_count == (\d+)\)", line)
        if m:
            cur["corners"] = int(m.group(1))
        m = re.search(r"return \((.*)\);", line)
        if m and "cells_label" in line:
            cur["lambda"] = m.group(1).strip()
        m = re.search(r"gt_sign_label = \{(.*)\};", line)
        if m:
            body = m.group(1).strip()
            cur["sign_label"] = [bool(int(x)) for x in body.split(",")] if body else []
        m = re.search(r"patch_gt = \{(.*)\};", line)
        if m:
            body = m.group(1).strip()
            if "std::pair" in line:
                pairs = re.findall(r"\{\s*(\d+)\s*,\s*(\d+)\s*\}", body)
                cur["patch_label"] = [[int(a), int(b)] for a, b in pairs]
            else:
                cur["patch_label"] = [int(x) for x in body.split(",")] if body else []
    out, csg = [], []
    for c in cases:
        tc = c["test_case"]
        if tc.startswith("implicit arrangement"):
            c["mode"] = "ia"
        elif tc.startswith("material interface on known"):
            c["mode"] = "mi"
        elif tc.startswith("CSG on known"):
            c["mode"] = "csg"
            c["positive_inside"] = True
            c["tree"] = lambda_to_tree(c["lambda"])
            csg.append(c)
            continue
        else:
            continue  # the failing example is not a known answer
        out.append(c)
    return out, csg


def lambda_to_tree(text: str):
    """The reference test's CSG lambda body (cells_label[i], !, &&, || and parentheses) as the units
    of a CSG tree file (app/csg.cpp:15-52): [op, a, b] with op 0 Intersection, 1 Union, 2 Negation;
    an element e > 0 is unit e (1-based), e < 0 is function -e-1; unit 1 is the root."""
    toks = re.findall(r"cells_label\[\d+\]|&&|\|\||!|\(|\)", text)
    if "".join(toks) != re.sub(r"\s+", "", text):
        raise ValueError("unsupported lambda: " + text)
    pos = 0

    def peek():
        return toks[pos] if pos < len(toks) else None

    def take():
        nonlocal pos
        pos += 1
        return toks[pos - 1]

    # expression tree first: ("f", j) | ("!", x) | ("&&"/"||", x, y)
    def expr():
        x = term()
        while peek() == "||":
            take()
            x = ("||", x, term())
        return x

    def term():
        x = factor()
        while peek() == "&&":
            take()
            x = ("&&", x, factor())
        return x

    def factor():
        t = take()
        if t == "!":
            return ("!", factor())
        if t == "(":
            x = expr()
            if take() != ")":
                raise ValueError("unbalanced parentheses: " + text)
            return x
        return ("f", int(re.search(r"\d+", t).group(0)))

    root = expr()
    if pos != len(toks):
        raise ValueError("trailing tokens: " + text)
    if root[0] == "f":
        root = ("||", root, root)
    units = []

    def emit(node):
        if node[0] == "f":
            return -node[1] - 1
        idx = len(units)
        units.append(None)
        if node[0] == "!":
            units[idx] = [2, emit(node[1]), 0]
        else:
            units[idx] = [0 if node[0] == "&&" else 1, emit(node[1]), emit(node[2])]
        return idx + 1

    emit(root)
    return units


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: python %s REFERENCE_ROOT" % sys.argv[0])
    ref = sys.argv[1]
    src_path = os.path.join(ref, "tests", "test_implicit_networks.cpp")
    with open(src_path) as f:
        kats, csg = parse_kats(f.read())
    for k in kats + csg:
        k["source"] = "tests/test_implicit_networks.cpp:%d" % k["line"]
    os.makedirs(os.path.join(HERE, "functions"), exist_ok=True)
    for name in sorted({k["functions"] for k in kats + csg}):
        shutil.copyfile(os.path.join(ref, "examples", "tests", name + ".json"),
                        os.path.join(HERE, "functions", name + ".json"))
    with open(os.path.join(ref, "examples", "tests", "mesh.json")) as f:
        mesh = json.load(f)
    np.savez_compressed(os.path.join(HERE, "mesh_8sphere.npz"),
                        pts=np.asarray(mesh[0], dtype=np.float64), tets=np.asarray(mesh[1], dtype=np.int64))
    with open(os.path.join(HERE, "kat.json"), "w") as f:
        json.dump(kats, f, indent=1)
    with open(os.path.join(HERE, "csg_kat.json"), "w") as f:
        json.dump(csg, f, indent=1)
    print("wrote %d known-answer cases and %d CSG known-answer cases" % (len(kats), len(csg)))


if __name__ == "__main__":
    main()
