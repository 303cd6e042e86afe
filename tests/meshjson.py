"""The reference's mesh.json (src/io.cpp:154-312) built from an oracle run, and helpers for the
C++ host-layer tests (test infrastructure)."""
import json

import numpy as np

KEYS = ["cells", "cells_label", "chains", "corners", "edges", "faces", "patches", "patches_label", "points",
        "shells"]


def _lists(offsets, items):
    out = [items[offsets[i]:offsets[i + 1]].tolist() for i in range(len(offsets) - 1)]
    return out or None


def expected_mesh_json(ref, mode):
    """mesh.json of the reference's writer for an oracle run with connectivity; cells, shells and
    cell labels are not built (null, or the MI writer's wrapped empty list)."""
    fo = ref["face_offsets"]
    faces = _lists(fo, ref["face_verts"])
    po = ref["patch_offsets"]  # both start with 0
    co = ref["chain_offsets"]
    edges = ref["edges"].tolist() or None
    corners = [i for i, d in enumerate(ref["nm_degree"].tolist()) if d == 1 or d > 2] or None
    if mode == "ia":
        plabel = [ref["patch_label"][:, 0].tolist()]
        clabel = None
    else:
        plabel = [ref["patch_label"].tolist()]
        clabel = [[]]
    return {
        "cells": None, "cells_label": clabel, "chains": _lists(co, ref["chain_edges"]), "corners": corners,
        "edges": edges, "faces": faces, "patches": _lists(po, ref["patch_faces"]), "patches_label": plabel,
        "points": ref["xyz"].tolist() or None, "shells": None,
    }


def nl_double(x):
    """A double as nlohmann-json prints it (shortest round-trip digits; fixed notation for decimal
    exponents -4 < n <= 15, else d.ddde+XX)."""
    x = float(x)
    if x != x or x in (float("inf"), float("-inf")):
        return "null"
    sign = "-" if str(x).startswith("-") else ""
    if x == 0.0:
        return sign + "0.0"
    s = repr(abs(x))
    m, ex = (s.split("e") + ["0"])[:2]
    ip, fp = (m.split(".") + [""])[:2]
    raw = ip + fp
    lead = len(raw) - len(raw.lstrip("0"))
    digits = raw.strip("0")
    n = len(ip) + int(ex) - lead
    k = len(digits)
    if k <= n <= 15:
        return sign + digits + "0" * (n - k) + ".0"
    if 0 < n <= 15:
        return sign + digits[:n] + "." + digits[n:]
    if -4 < n <= 0:
        return sign + "0." + "0" * (-n) + digits
    e = n - 1
    return sign + digits[0] + ("." + digits[1:] if k > 1 else "") + ("e-" if e < 0 else "e+") + "%02d" % abs(e)


def dump(v):
    """Compact JSON text with nlohmann's double format (keys already in order)."""
    if v is None:
        return "null"
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    if isinstance(v, float):
        return nl_double(v)
    if isinstance(v, dict):
        return "{" + ",".join('"%s":%s' % (k, dump(x)) for k, x in v.items()) + "}"
    return "[" + ",".join(dump(x) for x in v) + "]"


def load_mesh_json(path):
    with open(path) as f:
        text = f.read()
    d = json.loads(text)
    assert list(d) == KEYS, list(d)  # the reference's JSON library writes keys sorted
    assert text.endswith("}\n") and ": " not in text and ", " not in text  # compact dump + newline
    return d


def compare(got, exp, xyz_rtol=0.0):
    for k in KEYS:
        if k == "points" and exp[k] is not None and xyz_rtol > 0:
            a, b = np.asarray(got[k]), np.asarray(exp[k])
            assert a.shape == b.shape and np.all(np.abs(a - b) <= xyz_rtol * np.maximum(1.0, np.abs(b))), k
        else:
            assert got[k] == exp[k], k


def write_mesh_input(path, ref):
    """Input of `meshio_check mesh`: xyz, face offsets, face vertices, face function pairs."""
    with open(path, "wb") as f:
        for a, dt in ((ref["xyz"], np.float64), (ref["face_offsets"], np.int64), (ref["face_verts"], np.int64),
                      (ref["face_func"], np.int64)):
            a = np.ascontiguousarray(a, dtype=dt).ravel()
            f.write(np.int64(a.size).tobytes())
            f.write(a.tobytes())


def read_grid(path):
    with open(path, "rb") as f:
        buf = f.read()
    n = int(np.frombuffer(buf[:8], np.int64)[0])
    pts = np.frombuffer(buf[8:8 + 8 * n], np.float64).reshape(-1, 3)
    off = 8 + 8 * n
    m = int(np.frombuffer(buf[off:off + 8], np.int64)[0])
    tets = np.frombuffer(buf[off + 8:off + 8 + 8 * m], np.int64).reshape(-1, 4)
    return pts, tets
