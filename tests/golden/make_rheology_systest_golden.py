"""Collect the reference's rheology system tests into a small JSON fixture.

Reads, from the read-only reference tree (Underworld/Rheology/tests):
- input/testYieldCriterion.xml: the shared yield model (mesh resolution, box, wall velocities,
  background viscosity eta0, particle layout);
- input/testByerleeYieldCriterion.xml and input/testVonMisesYieldCriterion.xml: each yield law's
  parameters;
- expected/testByerleeYieldCriterion.expected and expected/testVonMisesYieldCriterion.expected:
  what the reference printed (time, step and the extent of the material points that yielded,
  each number with `%12.4g`);
- testNonNewtonianShear.xml, testNonNewtonianShearN3.0of1.sh, testNonNewtonianShearN4.0of1.sh and
  the expected/testNonNewtonianShearN{3,4}.0of1.*-ErrorFile.expected lines: the shear model (mesh,
  eta0, the stress exponents the two runs pass, the per-field tolerances and the non-linear
  tolerance) and which fields the reference found within tolerance of the analytic solution;
- NonNewtonianShearSolution/NonNewtonianShearSolution.c: the default top-wall velocity;
and writes tests/golden/rheology_systest_golden.json.  Run once with the reference tree's path as
the only argument; the fixture is committed.
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit(f"usage: python {os.path.basename(__file__)} <path of the Underworld 1.x source tree>")
REF = os.path.join(sys.argv[1], "Underworld/Rheology/tests")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rheology_systest_golden.json")


def _text(path):
    return re.sub(r"<!--.*?-->", "", open(path).read(), flags=re.S)


def params(path):
    """<param name="key"> value </param> entries of an input file (the last one of a name wins,
    as in the reference's dictionary merge)."""
    return {k: v.strip() for k, v in re.findall(r'<param name="([^"]+)"[^>]*>([^<]*)</param>', _text(path))}


def struct_params(path, name):
    body = re.search(r'<struct name="%s"[^>]*>(.*?)</struct>' % re.escape(name), _text(path), flags=re.S).group(1)
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

shear_xml = os.path.join(REF, "testNonNewtonianShear.xml")
s = params(shear_xml)
plugin = open(os.path.join(REF, "NonNewtonianShearSolution/NonNewtonianShearSolution.c")).read()
v_top = float(re.search(r'"velocityTopOfBox", ([-+0-9.eE]+)', plugin).group(1))
runs = {}
for tag in ("N3", "N4"):
    sh = open(os.path.join(REF, f"testNonNewtonianShear{tag}.0of1.sh")).read()
    n = float(re.search(r"--stressExponent=([0-9.]+)", sh).group(1))
    within = {}
    for field in ("VelocityField", "StrainRateField", "StressField", "ViscosityField"):
        txt = open(os.path.join(REF, "expected", f"testNonNewtonianShear{tag}.0of1.{field}-ErrorFile.expected")).read()
        within[field] = [int(t) for t in re.findall(r"Timestep (\d+): [^\n]* is within a tolerance", txt)]
    runs[tag] = {"stressExponent": n, "within": within}
shear = {
    "elementRes": [int(s["elementResI"]), int(s["elementResJ"])],
    "min": [float(s["minX"]), float(s["minY"])],
    "max": [float(s["maxX"]), float(s["maxY"])],
    "eta0": float(struct_params(shear_xml, "layerViscosity")["eta0"]),
    "gaussParticles": [int(s["gaussParticlesX"]), int(s["gaussParticlesY"])],
    "velocityTopOfBox": v_top,
    "nonLinearTolerance": float(s["nonLinearTolerance"]),
    "tolerance": {f: float(s[f + "-Tolerance"]) for f in ("VelocityField", "StrainRateField", "StressField",
                                                           "ViscosityField")},
    "runs": runs,
}
json.dump({"model": model, "laws": laws, "nonNewtonianShear": shear}, open(OUT, "w"), indent=1)
print(OUT)
