"""Regenerate the paper-example fixtures in examples/ from the reference checkout.

Reads, as data, the function files and configs of
  * examples/Fig19_teaser_left/<model>/: inverse-CSG models of 16 to 26 planes, cylinders and tori
    (implicit arrangement);
  * examples/Fig16/{IA,MI}/with_*_look_up/: 18 spheres (implicit arrangement and material
    interface; the reference's secondary-lookup ablation runs the same file with the switch off).
Writes examples/<name>.json (the function list) and examples/manifest.json (mode, grid resolution,
box and lookup switches of each).

Usage: python tests/golden/make_examples.py REFERENCE_ROOT
Nothing else reads the reference checkout; the tests only read the files written here.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def entry(src_dir, name, mode, out_dir):
    cfg = json.load(open(os.path.join(src_dir, "config.json")))
    funcs = json.load(open(os.path.join(src_dir, os.path.basename(cfg["funcFile"]))))
    with open(os.path.join(out_dir, name + ".json"), "w") as f:
        json.dump(funcs, f, indent=1)
    return {"file": name + ".json", "mode": mode, "resolution": int(cfg["gridResolution"]),
            "bbox": cfg.get("gridBbox", [[-1, -1, -1], [1, 1, 1]]),
            "use_lookup": bool(cfg.get("useLookup", True)),
            "use_secondary_lookup": bool(cfg.get("useSecondaryLookup", True))}


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: python %s REFERENCE_ROOT" % sys.argv[0])
    root = sys.argv[1]
    ex = os.path.join(root, "examples")
    out_dir = os.path.join(HERE, "examples")
    os.makedirs(out_dir, exist_ok=True)
    manifest = []
    fig19 = os.path.join(ex, "Fig19_teaser_left")
    for model in sorted(os.listdir(fig19), key=int):
        manifest.append(entry(os.path.join(fig19, model), "fig19_csg_%s" % model, "ia", out_dir))
    manifest.append(entry(os.path.join(ex, "Fig16", "IA", "with_2func_look_up"), "fig16_ia_18sphere", "ia", out_dir))
    manifest.append(entry(os.path.join(ex, "Fig16", "MI", "with_3func_look_up"), "fig16_mi_18sphere", "mi", out_dir))
    with open(os.path.join(out_dir, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("wrote %d fixtures to %s" % (len(manifest), out_dir))


if __name__ == "__main__":
    main()
