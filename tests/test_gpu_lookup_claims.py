"""The secondary lookup without its seeded table (RIA_NO_LOOKUP_SEED, read when a process builds its
tables): every key is claimed by the first tet that sees it, cut once, published, and taken by the
key's other tets after the cuts.  Results equal the general cut and the oracle, on the first call
(all keys claimed) and the second (all published), for both modes."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
sys.path[:0] = [{repo!r}, {repo!r} + "/oracle", {repo!r} + "/tests"]
import importlib
import numpy as np
import pyoracle
from test_gpu_ia import assert_mesh_equal
pkg = importlib.import_module("robust-implicit-surface-networks_gb300")
fns = importlib.import_module("robust-implicit-surface-networks_gb300.functions")
pkg.build(); pyoracle.build()
for mode in ("ia", "mi"):
    wl = fns.workload_ia_degenerate(res=36) if mode == "ia" else fns.workload_mi(res=36)
    grid = pkg.grid_implicit_arrangement if mode == "ia" else pkg.grid_material_interface
    pts, tets = fns.generate_tet_mesh(wl.res)
    ref = pyoracle.run(mode, pts, tets, pyoracle.sample(wl.funcs, pts))
    off = grid(wl.res, wl.funcs, use_secondary_lookup=False)
    for it in range(2):
        on = grid(wl.res, wl.funcs, use_secondary_lookup=True)
        assert_mesh_equal(on, ref)
        for k in ("rec_bytes", "verts", "face_verts", "xyz"):
            assert np.array_equal(on[k], off[k]), (mode, it, k)
    pkg.load().ria_lookup_cache_clear()
    on = grid(wl.res, wl.funcs, use_secondary_lookup=True)
    assert np.array_equal(on["rec_bytes"], off["rec_bytes"]), (mode, "after reset")
print("ok")
"""


def test_claims_without_seeded_table():
    env = dict(os.environ, RIA_NO_LOOKUP_SEED="1")
    r = subprocess.run([sys.executable, "-c", SCRIPT.format(repo=REPO)], env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-2000:] + r.stderr[-4000:]
