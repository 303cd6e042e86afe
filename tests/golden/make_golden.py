"""Regenerate the golden fixtures in this folder from the reference checkout.

Reads, as data:
  * the known-answer tests of tests/test_implicit_networks.cpp (TEST_CASE / SECTION blocks:
    the function file, the tet mesh, and the REQUIREd patch count, chain count, corner count and
    patch_function_label list);
  * the function lists examples/tests/*.json and the tet mesh examples/tests/mesh.json.
Writes kat.json, functions/*.json and mesh_8sphere.npz next to this script.

Usage: python tests/golden/make_golden.py [reference_root]
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
        m = re.search(r"patch_gt = \{(.*)\};", line)
        if m:
            body = m.group(1).strip()
            if "std::pair" in line:
                pairs = re.findall(r"\{\s*(\d+)\s*,\s*(\d+)\s*\}", body)
                cur["patch_label"] = [[int(a), int(b)] for a, b in pairs]
            else:
                cur["patch_label"] = [int(x) for x in body.split(",")] if body else []
    out = []
    for c in cases:
        tc = c["test_case"]
        if tc.startswith("implicit arrangement"):
            c["mode"] = "ia"
        elif tc.startswith("material interface on known"):
            c["mode"] = "mi"
        else:
            continue  # CSG needs arrangement cells; the failing example is not a known answer
        out.append(c)
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    src_path = os.path.join(ref, "tests", "test_implicit_networks.cpp")
    with open(src_path) as f:
        kats = parse_kats(f.read())
    for k in kats:
        k["source"] = "tests/test_implicit_networks.cpp:%d" % k["line"]
    os.makedirs(os.path.join(HERE, "functions"), exist_ok=True)
    for name in sorted({k["functions"] for k in kats}):
        shutil.copyfile(os.path.join(ref, "examples", "tests", name + ".json"),
                        os.path.join(HERE, "functions", name + ".json"))
    with open(os.path.join(ref, "examples", "tests", "mesh.json")) as f:
        mesh = json.load(f)
    np.savez_compressed(os.path.join(HERE, "mesh_8sphere.npz"),
                        pts=np.asarray(mesh[0], dtype=np.float64), tets=np.asarray(mesh[1], dtype=np.int64))
    with open(os.path.join(HERE, "kat.json"), "w") as f:
        json.dump(kats, f, indent=1)
    print("wrote %d known-answer cases" % len(kats))


if __name__ == "__main__":
    main()
