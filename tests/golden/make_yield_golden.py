"""Collect the reference's yield-criterion system tests into a small JSON fixture.

Reads, from the read-only reference tree:
- Underworld/Rheology/tests/input/testYieldCriterion.xml: the shared model (mesh resolution, box,
  wall velocities, background viscosity eta0, particle layout);
- Underworld/Rheology/tests/input/testByerleeYieldCriterion.xml and
  testVonMisesYieldCriterion.xml: each yield law's parameters;
- Underworld/Rheology/tests/expected/testByerleeYieldCriterion.expected and
  testVonMisesYieldCriterion.expected: what the reference printed (time, step and the extent of
  the material points that yielded, each number with `%12.4g`);
and writes tests/golden/yield_golden.json.  Run once with the reference tree's path as the only
argument; the fixture is committed.
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit(f"usage: python {os.path.basename(__file__)} <path of the Underworld 1.x source tree>")
REF = os.path.join(sys.argv[1], "Underworld/Rheology/tests")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "yield_golden.json")


def params(path):
    """<param name="key"> value </param> entries of an input file (the last one of a name wins,
    as in the reference's dictionary merge)."""
    txt = re.sub(r"<!--.*?-->", "", open(path).read(), flags=re.S)
    return {k: v.strip() for k, v in re.findall(r'<param name="([^"]+)"[^>]*>([^<]*)</param>', txt)}


def struct_params(path, name):
    txt = re.sub(r"<!--.*?-->", "", open(path).read(), flags=re.S)
    body = re.search(r'<struct name="%s"[^>]*>(.*?)</struct>' % re.escape(name), txt, flags=re.S).group(1)
    return {k: v.strip() for k, v in re.findall(r'<param name="([^"]+)"[^>]*>([^<]*)</param>', body)}


def expected(path):
    txt = open(path).read()
    head = re.search(r"Material yielded at time\s+(\S+) \(step (\d+)\) within:", txt)
    ext = {ax: re.search(r"%s:\s+(\S+)\s+-\s+(\S+)" % ax, txt).groups() for ax in "xy"}
    return {"time": head.group(1), "step": int(head.group(2)), "x": list(ext["x"]), "y": list(ext["y"])}


base = os.path.join(REF, "input/testYieldCriterion.xml")
p = params(base)
model = {
    "elementRes": [int(p["elementResI"]), int(p["elementResJ"])],
    "min": [float(p["minX"]), float(p["minY"])],
    "max": [float(p["maxX"]), float(p["maxY"])],
    "leftWallVelocity": float(p["leftWallVelocity"]),
    "rightWallVelocity": float(p["rightWallVelocity"]),
    "eta0": float(struct_params(base, "layerViscosity")["eta0"]),
    "particleLayout": struct_params(base, "materialSwarmParticleLayout")["Type"],
}
laws = {}
for law, fname in (("Byerlee", "testByerleeYieldCriterion"), ("VonMises", "testVonMisesYieldCriterion")):
    y = struct_params(os.path.join(REF, "input", fname + ".xml"), "yieldRheology")
    assert y["Type"] == law, y
    laws[law] = {
        "cohesion": float(y["cohesion"]),
        "depthCoefficient": float(y.get("depthCoefficient", 0.0)),
        "expected": expected(os.path.join(REF, "expected", fname + ".expected")),
    }
json.dump({"model": model, "laws": laws}, open(OUT, "w"), indent=1)
print(OUT)
