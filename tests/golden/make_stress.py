"""Regenerate the near-degenerate stress fixtures in stress/ from the reference checkout.

Reads, as data, the robustness sets examples/Table2_Fig11/{IA,MI}/<noise>/<id>/{config,functions}.json:
four spheres whose centres differ by about `noise` (implicit arrangement) and five functions of
spheres and zeros (material interface), sampled on a grid of gridResolution cubes per axis.  Keeps
the first `per_level` instances of every noise level (by instance number) and writes
stress/<mode>_<noise>_<id>.json (the function list) and stress/manifest.json (mode, noise, instance,
grid resolution and box of each).

Usage: python tests/golden/make_stress.py REFERENCE_ROOT [per_level]
Nothing else reads the reference checkout; the tests only read the files written here.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: python %s REFERENCE_ROOT" % sys.argv[0])
    root = sys.argv[1]
    per_level = int(sys.argv[2]) if len(sys.argv) > 2 else 3
    base = os.path.join(root, "examples", "Table2_Fig11")
    out_dir = os.path.join(HERE, "stress")
    os.makedirs(out_dir, exist_ok=True)
    manifest = []
    for mode in ("IA", "MI"):
        for noise in sorted(os.listdir(os.path.join(base, mode)), key=float):
            ids = sorted((d for d in os.listdir(os.path.join(base, mode, noise)) if d.isdigit()), key=int)
            for inst in ids[:per_level]:
                src = os.path.join(base, mode, noise, inst)
                cfg = json.load(open(os.path.join(src, "config.json")))
                funcs = json.load(open(os.path.join(src, "functions.json")))
                name = "%s_%s_%s.json" % (mode.lower(), noise, inst)
                with open(os.path.join(out_dir, name), "w") as f:
                    json.dump(funcs, f, indent=1)
                manifest.append({"file": name, "mode": mode.lower(), "noise": noise, "instance": int(inst),
                                 "resolution": int(cfg["gridResolution"]),
                                 "bbox": cfg.get("gridBbox", [[-1, -1, -1], [1, 1, 1]])})
    with open(os.path.join(out_dir, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("wrote %d fixtures to %s" % (len(manifest), out_dir))


if __name__ == "__main__":
    main()
