"""Generate tests/golden/known_answers.json from the reference's own test files and docs.

The reference's CPU known-answer tests and published layout sizes are read as text from a
checkout of erw-1/d3-force-3d-webgpu and written out as small fixtures, so that the GPU machine
(which has no copy of the reference) can check the oracle against them.

    python tests/golden/make_golden.py <path of the reference checkout>

Sources (paths within the reference):
  test/simulation-test.js:10-17   phyllotaxis start of three 2D nodes
  test/center-test.js:4-22        forceCenter on three nodes, and with a pinned node
  test/collide-test.js:5-50       forceCollide after 10 + 10 ticks; coincident-node jiggle
  docs/differences.md:35-40       RMS layout radius after 300 ticks, 1,000-node random graph
  examples/benchmark.html:86-93   the graph generator those sizes come from (seed 42)
"""
import json
import os
import re
import sys


def node_values(text):
    """Every `assertNodeEqual(name, {...})` object literal, as dicts of numbers."""
    out = []
    for m in re.finditer(r"assertNodeEqual\((\w+(?:\[\d+\])?),\s*\{([^}]*)\}\)", text):
        fields = {}
        for k, v in re.findall(r"(\w+):\s*(-?[\d.eE+-]+)", m.group(2)):
            fields[k] = float(v)
        out.append({"node": m.group(1), "expect": fields})
    return out


def main(ref):
    rd = lambda p: open(os.path.join(ref, p)).read()
    sim = rd("test/simulation-test.js")
    center = rd("test/center-test.js")
    collide = rd("test/collide-test.js")
    diffs = rd("docs/differences.md")

    # docs/differences.md table: "| 3D, CPU | 372 | 418 | 499 | 548 |"
    sizes = {}
    for dims, side, vals in re.findall(r"\|\s*(\d)D, (CPU|GPU)\s*\|([^\n]*)", diffs):
        nums = [float(x) for x in re.findall(r"\d+", vals)]
        sizes["%sD_%s" % (dims, side)] = nums
    thetas = [0.9, 0.5, 0.2, 0.0]

    golden = {
        "source": "erw-1/d3-force-3d-webgpu test/*.js and docs/differences.md, read as text",
        "tolerance_abs": 1e-6,  # test/asserts.js:3-15
        "phyllotaxis_2d": node_values(sim),
        "center": node_values(center),
        "collide": node_values(collide),
        "layout_rms_radius": {"thetas": thetas, "nodes": 1000, "ticks": 300,
                              "link_distance": 30, "graph_seed": 42, "values": sizes},
    }
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "known_answers.json")
    with open(out, "w") as f:
        json.dump(golden, f, indent=1)
    print("wrote", out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the erw-1/d3-force-3d-webgpu checkout>")
    main(sys.argv[1])
