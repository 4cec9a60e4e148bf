"""Generate the numbering golden fixtures by running the SeismoVLAB
pre-processor itself (PP/Method/Builder.py makeDomainArea/Volume, the
Attach.py builders and PP/Core/Numberer.py PlainScheme via
CreateRunAnalysisFiles) on small structured models, and keeping the
partition file's node dof numbers, connectivity and constraints.

Run from the repository root where the reference tree is available:
    python tests/golden/make_numbering_fixtures.py /path/to/SVL
The reference imports matplotlib, which is not installed here; a stub module
is written to a scratch folder for the subprocesses.  Outputs:
tests/golden/numbering_<case>.json.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent

CASES = {
    # config-1 style box: fixed bottom, x-roller sides (Q4)
    "q4_box": dict(ndim=2, ne=[6, 4], h=[1.0, 1.0], fix=[(0, [1]), (1, [1]), (2, [1, 2])], periodic=False),
    # config-3 style soil column: fixed base, periodic sides via EQUAL constraints (Q4)
    "q4_column_periodic": dict(ndim=2, ne=[3, 5], h=[0.5, 0.5], fix=[(2, [1, 2])], periodic=True),
    # config-2/4 style box: fixed bottom, rollers on the four sides (H8)
    "h8_box": dict(ndim=3, ne=[3, 2, 2], h=[2.0, 2.0, 2.0],
                   fix=[(0, [1]), (1, [1]), (2, [2]), (3, [2]), (4, [1, 2, 3])], periodic=False),
}

DRIVER = r'''
import json, sys
import numpy as np
from Core import SeismoVLAB as SVL
case = json.loads(sys.argv[1])
nd = case["ndim"]; ne = case["ne"]; h = case["h"]
SVL.Options["file"] = "Fixture"
SVL.Options["nparts"] = 1
SVL.Options["dimension"] = nd
SVL.Options["massform"] = "lumped"
if nd == 2:
    SVL.addMaterial(tag=1, name="Elastic2DPlaneStrain", attributes={"E": 2.0e8, "nu": 0.25, "rho": 2000.0})
    mesh = SVL.makeDomainArea(options={"ne": ne, "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
        "P0": [0.0, 0.0], "P1": [ne[0]*h[0], 0.0], "P2": [0.0, ne[1]*h[1]],
        "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
else:
    SVL.addMaterial(tag=1, name="Elastic3DLinear", attributes={"E": 2.0e8, "nu": 0.25, "rho": 2000.0})
    mesh = SVL.makeDomainVolume(options={"ne": ne, "ndof": 3, "class": "LIN3DHEXA8", "elems": "HEXA8",
        "P0": [0.0, 0.0, 0.0], "P1": [ne[0]*h[0], 0.0, 0.0], "P2": [0.0, ne[1]*h[1], 0.0], "P3": [0.0, 0.0, ne[2]*h[2]],
        "attributes": {"material": 1, "rule": "Gauss", "np": 8}})
for tag in sorted(mesh["Nodes"]):
    n = mesh["Nodes"][tag]
    SVL.addNode(tag=tag, ndof=n["ndof"], coords=list(map(float, n["coords"])))
for tag in sorted(mesh["Elements"]):
    el = mesh["Elements"][tag]
    SVL.addElement(tag=tag, conn=list(el["conn"]), name=el["name"], attributes=dict(el["attributes"]))
nx, ny = ne[0], ne[1]; nz = ne[2] if nd == 3 else 0
def ijk(tag):
    t = tag - 1
    i = t % (nx + 1); j = (t // (nx + 1)) % (ny + 1); k = t // ((nx + 1) * (ny + 1)) if nd == 3 else 0
    return i, j, k
faces = {0: lambda i,j,k: i == 0, 1: lambda i,j,k: i == nx, 2: lambda i,j,k: j == 0, 3: lambda i,j,k: j == ny,
         4: lambda i,j,k: nd == 3 and k == 0, 5: lambda i,j,k: nd == 3 and k == nz}
if nd == 2:
    faces = {0: faces[0], 1: faces[1], 2: faces[2], 3: faces[3]}
for f, dofs in case["fix"]:
    for tag in sorted(mesh["Nodes"]):
        if faces[f](*ijk(tag)):
            SVL.addRestrain(tag=tag, dof=list(dofs))
ctag = -2
if case["periodic"]:
    for tag in sorted(mesh["Nodes"]):
        i, j, k = ijk(tag)
        if i != nx:
            continue
        master = tag - nx
        for d in range(nd):
            if SVL.Entities["Nodes"][tag]["freedof"][d] == -1:
                continue
            SVL.addConstraint(tag=ctag, name="Equal", attributes={"stag": tag, "sdof": d + 1, "mtag": [master], "mdof": [d + 1]})
            ctag -= 1
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "series.txt", "dir": [0.0] * (nd - 1) + [-1.0]})
SVL.addLoad(tag=1, name="PointLoad", attributes={"type": "Concentrated", "fun": 1, "list": [max(mesh["Nodes"])]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [1.0]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": 3})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "CentralDifference", "dt": 1e-3})
SVL.addSolver(tag=1, attributes={"name": "Eigen", "update": "OFF"})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
'''


def main(ref_root: str):
    ref = Path(ref_root)
    pp = ref / "01-Pre_Process"
    scratch = HERE / ".pp_scratch"
    if scratch.exists():
        shutil.rmtree(scratch)
    stub = scratch / "stub" / "matplotlib"
    stub.mkdir(parents=True)
    (stub / "__init__.py").write_text("def use(*a, **k):\n    pass\n")
    for mod in ("pyplot.py", "pylab.py"):
        (stub / mod).write_text("def __getattr__(name):\n    return lambda *a, **k: None\n")
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([str(scratch / "stub"), str(pp)]))
    for name, case in CASES.items():
        work = scratch / name
        work.mkdir(parents=True)
        (work / "series.txt").write_text("3\n0.0\n1.0\n0.0\n")
        r = subprocess.run([sys.executable, "-c", DRIVER, json.dumps(case)], cwd=work, env=env,
                           capture_output=True, text=True, timeout=300)
        if r.returncode != 0:
            raise SystemExit("pre-processor failed for %s:\n%s\n%s" % (name, r.stdout, r.stderr))
        part = next((work / "Partition").glob("*.json"))
        data = json.loads(part.read_text())
        tags = sorted(int(t) for t in data["Nodes"])
        etags = sorted(int(t) for t in data["Elements"])
        out = {
            "case": case,
            "generated_by": "SeismoVLAB pre-processor (PP/Core/Numberer.py PlainScheme) via tests/golden/make_numbering_fixtures.py",
            "ntotal": data["Global"]["ntotal"], "nfree": data["Global"]["nfree"],
            "node_tags": tags,
            "freedof": [data["Nodes"][str(t)]["freedof"] for t in tags],
            "totaldof": [data["Nodes"][str(t)]["totaldof"] for t in tags],
            "coords": [data["Nodes"][str(t)]["coords"] for t in tags],
            "elem_tags": etags,
            "conn": [data["Elements"][str(t)]["conn"] for t in etags],
            "constraints": {k: v for k, v in sorted(data.get("Constraints", {}).items(), key=lambda kv: -int(kv[0]))},
        }
        (HERE / ("numbering_%s.json" % name)).write_text(json.dumps(out, separators=(",", ":")) + "\n")
        print("wrote numbering_%s.json (%d nodes, ntotal=%d, nfree=%d)" % (name, len(tags), out["ntotal"], out["nfree"]))
    shutil.rmtree(scratch)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SVL_REFERENCE_ROOT")
    if not root:
        raise SystemExit("usage: %s <SVL source tree>  (or set SVL_REFERENCE_ROOT)" % Path(__file__).name)
    main(root)
