"""Regenerates the golden fixtures in this folder from the SyFrack source tree.

Run in a checkout that has the reference next to it:
    python tests/golden/make_golden.py /path/to/SyFrack
It reads, as data:
  crates/syfrack-core/tests/fixtures/parity/{sphere,mandelbulb,mandelbox,menger}.ron
      -> de_parity_<name>.json  (64 LCG points, distance, traps, iterations;
         the samples graph_parity.rs checks the bundled graphs against)
  graphs/{sphere,mandelbulb,mandelbox,menger}.ron
      -> graph_<name>.json      (nodes, links, safety, bounding_radius_hint)
The JSON files are committed; nothing at test time reads the reference.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from syfrack_gb300 import ron  # noqa: E402

NAMES = ["sphere", "mandelbulb", "mandelbox", "menger"]
EXTENTS = {"sphere": 3.0, "mandelbulb": 1.6, "mandelbox": 8.0, "menger": 1.6}


def to_json(v):
    if isinstance(v, ron.Unit):
        return v.name
    if isinstance(v, ron.Tuple):
        return [to_json(x) for x in v.items]
    if isinstance(v, dict):
        return {k: to_json(x) for k, x in v.items()}
    if isinstance(v, list):
        return [to_json(x) for x in v]
    return v


def main(root):
    for name in NAMES:
        fx = ron.load(os.path.join(root, "crates/syfrack-core/tests/fixtures/parity", f"{name}.ron"))
        rows = [{"p": ron.vec(r["p"]), "distance": r["distance"], "traps": ron.vec(r["traps"]),
                 "iterations": r["iterations"]} for r in fx]
        with open(os.path.join(HERE, f"de_parity_{name}.json"), "w") as f:
            json.dump({"source": f"crates/syfrack-core/tests/fixtures/parity/{name}.ron",
                       "extent": EXTENTS[name], "lcg_seed": 11, "samples": rows}, f, indent=0)
        g = ron.load(os.path.join(root, "graphs", f"{name}.ron"))
        with open(os.path.join(HERE, f"graph_{name}.json"), "w") as f:
            json.dump({"source": f"graphs/{name}.ron", "graph": to_json(g)}, f, indent=1)
    print("wrote", len(NAMES) * 2, "files")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
