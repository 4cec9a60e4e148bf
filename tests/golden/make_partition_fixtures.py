"""Generate complete SVL partition files (and their time-series files) by
running the SeismoVLAB pre-processor itself (PP/Core/SeismoVLAB.py
CreateRunAnalysisFiles) on small models that exercise every field the
partition reader maps: materials (elastic and J2), restraints, EQUAL
constraints, point and element body loads (constant and time series),
support motions, Rayleigh dampings, PML layers, Lysmer dashpots,
domain-reduction loads, node recorders, the integrator/algorithm/solver
settings.

Run from the repository root where the reference tree is available:
    python tests/golden/make_partition_fixtures.py /path/to/SVL
The reference imports matplotlib, which is not installed here; a stub module
is written to a scratch folder for the subprocesses.  Outputs:
tests/golden/partition_<case>/ with the partition JSON under Partition/ and
the time-series files next to it (the run directory layout of the reference).
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent

COMMON = r'''
import json, sys, math
import numpy as np
from Core import SeismoVLAB as SVL
case = sys.argv[1]
SVL.Options["file"] = "Fixture"
SVL.Options["nparts"] = 1
def ricker(nt, dt, f0, amp):
    t0 = 1.2 / f0
    out = []
    for k in range(nt):
        b = (math.pi * f0 * (k * dt - t0)) ** 2
        out.append(amp * (1 - 2 * b) * math.exp(-b))
    return out
def write_series(name, vals):
    with open(name, "w") as f:
        f.write("%d\n" % len(vals))
        for v in vals:
            f.write("%.17g\n" % v)
'''

CASES = {
    # Q4 elastic box, point load time series + constant point load, CD, node recorder
    "q4_cd": COMMON + r'''
SVL.Options["dimension"] = 2
SVL.Options["massform"] = "lumped"
nx, ny, dt, nt = 6, 4, 1.0e-3, 41
SVL.addMaterial(tag=1, name="Elastic2DPlaneStrain", attributes={"E": 2.0e8, "nu": 0.25, "rho": 2000.0})
SVL.addMaterial(tag=2, name="Elastic2DPlaneStrain", attributes={"E": 3.0e8, "nu": 0.30, "rho": 2100.0})
mesh = SVL.makeDomainArea(options={"ne": [nx, ny], "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
    "P0": [0.0, 0.0], "P1": [nx * 1.0, 0.0], "P2": [0.0, ny * 1.0],
    "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
for tag in sorted(mesh["Nodes"]):
    n = mesh["Nodes"][tag]
    SVL.addNode(tag=tag, ndof=n["ndof"], coords=list(map(float, n["coords"])))
for tag in sorted(mesh["Elements"]):
    el = mesh["Elements"][tag]
    at = dict(el["attributes"])
    if tag % 3 == 0:
        at["material"] = 2
    SVL.addElement(tag=tag, conn=list(el["conn"]), name=el["name"], attributes=at)
for tag in sorted(mesh["Nodes"]):
    t = tag - 1; i = t % (nx + 1); j = t // (nx + 1)
    if j == 0:
        SVL.addRestrain(tag=tag, dof=[1, 2])
    elif i == 0 or i == nx:
        SVL.addRestrain(tag=tag, dof=1)
write_series("ricker.txt", ricker(nt, dt, 25.0, 1.0e5))
top = ny * (nx + 1) + nx // 2 + 1
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "ricker.txt", "dir": [0.0, -1.0]})
SVL.addFunction(tag=2, name="Constant", attributes={"mag": 2.5e3, "dir": [1.0, 0.0]})
SVL.addLoad(tag=1, name="PointLoad", attributes={"type": "Concentrated", "fun": 1, "list": [top]})
SVL.addLoad(tag=2, name="PointLoad", attributes={"type": "Concentrated", "fun": 2, "list": [top - 1]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1, 2], "factor": [1.0, 0.5]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Disp.out", "ndps": 8, "resp": "disp", "list": [top, top - 1]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "CentralDifference", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Eigen", "update": "OFF"})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # Q4 box with nodal masses and a body point load (acceleration times the
    # node's mass) beside a concentrated load on the same node, CD
    "q4_bodypoint_cd": COMMON + r'''
SVL.Options["dimension"] = 2
SVL.Options["massform"] = "lumped"
nx, ny, dt, nt = 6, 4, 1.0e-3, 41
SVL.addMaterial(tag=1, name="Elastic2DPlaneStrain", attributes={"E": 2.0e8, "nu": 0.25, "rho": 2000.0})
mesh = SVL.makeDomainArea(options={"ne": [nx, ny], "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
    "P0": [0.0, 0.0], "P1": [nx * 1.0, 0.0], "P2": [0.0, ny * 1.0],
    "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
for tag in sorted(mesh["Nodes"]):
    n = mesh["Nodes"][tag]
    SVL.addNode(tag=tag, ndof=n["ndof"], coords=list(map(float, n["coords"])))
for tag in sorted(mesh["Elements"]):
    el = mesh["Elements"][tag]
    SVL.addElement(tag=tag, conn=list(el["conn"]), name=el["name"], attributes=dict(el["attributes"]))
for tag in sorted(mesh["Nodes"]):
    t = tag - 1; i = t % (nx + 1); j = t // (nx + 1)
    if j == 0:
        SVL.addRestrain(tag=tag, dof=[1, 2])
    elif i == 0 or i == nx:
        SVL.addRestrain(tag=tag, dof=1)
top = ny * (nx + 1) + nx // 2 + 1
SVL.addMass(tag=top, dof=[1, 2], vals=[250.0, 400.0])
SVL.addMass(tag=top - 1, dof=[1, 2], vals=[120.0, 120.0])
write_series("accel.txt", ricker(nt, dt, 25.0, 40.0))
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "accel.txt", "dir": [0.6, -0.8]})
SVL.addFunction(tag=2, name="Constant", attributes={"mag": 2.0e3, "dir": [1.0, 0.0]})
SVL.addLoad(tag=1, name="PointLoad", attributes={"type": "Body", "fun": 1, "list": [top, top - 1, top + 1]})
SVL.addLoad(tag=2, name="PointLoad", attributes={"type": "Concentrated", "fun": 2, "list": [top]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1, 2], "factor": [1.0, 0.5]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Disp.out", "ndps": 8, "resp": "disp", "list": [top, top - 1]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "CentralDifference", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Eigen", "update": "OFF"})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # H8 elastic box, element body load time series, Newmark + PETSc CG
    "h8_newmark_body": COMMON + r'''
SVL.Options["dimension"] = 3
SVL.Options["massform"] = "lumped"
nx, ny, nz, dt, nt = 3, 3, 2, 2.0e-3, 31
SVL.addMaterial(tag=1, name="Elastic3DLinear", attributes={"E": 2.0e8, "nu": 0.3, "rho": 2000.0})
mesh = SVL.makeDomainVolume(options={"ne": [nx, ny, nz], "ndof": 3, "class": "LIN3DHEXA8", "elems": "HEXA8",
    "P0": [0.0, 0.0, 0.0], "P1": [nx * 2.0, 0.0, 0.0], "P2": [0.0, ny * 2.0, 0.0], "P3": [0.0, 0.0, nz * 2.0],
    "attributes": {"material": 1, "rule": "Gauss", "np": 8}})
for tag in sorted(mesh["Nodes"]):
    n = mesh["Nodes"][tag]
    SVL.addNode(tag=tag, ndof=n["ndof"], coords=list(map(float, n["coords"])))
for tag in sorted(mesh["Elements"]):
    el = mesh["Elements"][tag]
    SVL.addElement(tag=tag, conn=list(el["conn"]), name=el["name"], attributes=dict(el["attributes"]))
for tag in sorted(mesh["Nodes"]):
    t = tag - 1; k = t // ((nx + 1) * (ny + 1))
    if k == 0:
        SVL.addRestrain(tag=tag, dof=[1, 2, 3])
write_series("body.txt", ricker(nt, dt, 20.0, 1.0))
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "body.txt", "dir": [1.0, 0.0, 0.0]})
SVL.addLoad(tag=1, name="ElementLoad", attributes={"type": "Body", "fun": 1, "list": [8, 11]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [2.0e3]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Disp.out", "ndps": 10, "resp": "disp", "list": [40, 48]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "Newmark", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Petsc", "option": "KSPCG", "tol": 1.0e-10})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # J2 soil column: periodic sides (EQUAL constraints), base support motion, CD
    "q4_j2_column": COMMON + r'''
SVL.Options["dimension"] = 2
SVL.Options["massform"] = "lumped"
nx, ny, h, dt, nt = 2, 6, 0.5, 2.0e-4, 61
G = 2000.0 * 200.0 ** 2; K = 2 * G * 1.3 / (3 * 0.4)
SVL.addMaterial(tag=1, name="PlasticPlaneStrainJ2", attributes={"K": K, "G": G, "rho": 2000.0, "h": 0.02 * G,
                                                                 "beta": 1.0, "Sy": math.sqrt(3.0) * 40.0e3})
mesh = SVL.makeDomainArea(options={"ne": [nx, ny], "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
    "P0": [0.0, 0.0], "P1": [nx * h, 0.0], "P2": [0.0, ny * h],
    "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
for tag in sorted(mesh["Nodes"]):
    n = mesh["Nodes"][tag]
    SVL.addNode(tag=tag, ndof=n["ndof"], coords=list(map(float, n["coords"])))
for tag in sorted(mesh["Elements"]):
    el = mesh["Elements"][tag]
    SVL.addElement(tag=tag, conn=list(el["conn"]), name=el["name"], attributes=dict(el["attributes"]))
base = [t for t in sorted(mesh["Nodes"]) if (t - 1) // (nx + 1) == 0]
for tag in base:
    SVL.addRestrain(tag=tag, dof=[1, 2])
ctag = -2
for tag in sorted(mesh["Nodes"]):
    i = (tag - 1) % (nx + 1)
    if i != nx or tag in base:
        continue
    for d in range(2):
        SVL.addConstraint(tag=ctag, name="Equal", attributes={"stag": tag, "sdof": d + 1, "mtag": [tag - nx], "mdof": [d + 1]})
        ctag -= 1
motion = [0.02 * math.sin(2 * math.pi * 8.0 * k * dt) * (1 - math.exp(-k / 10.0)) for k in range(nt)]
write_series("base.txt", motion)
for tag in base:
    SVL.addSupportMotion(tag=tag, attributes={"type": "TimeSeries", "file": "base.txt", "dof": 1})
SVL.addFunction(tag=1, name="Constant", attributes={"mag": 0.0, "dir": [0.0, -1.0]})
SVL.addLoad(tag=1, name="PointLoad", attributes={"type": "Concentrated", "fun": 1, "list": [max(mesh["Nodes"])]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [1.0]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Top.out", "ndps": 8, "resp": "disp", "list": [max(mesh["Nodes"])]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "CentralDifference", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Eigen", "update": "OFF"})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # Q4 box with two Rayleigh dampings over element groups, Newmark + PETSc CG
    "q4_newmark_rayleigh": COMMON + r'''
SVL.Options["dimension"] = 2
SVL.Options["massform"] = "lumped"
nx, ny, dt, nt = 6, 4, 2.0e-3, 31
SVL.addMaterial(tag=1, name="Elastic2DPlaneStrain", attributes={"E": 2.0e8, "nu": 0.25, "rho": 2000.0})
mesh = SVL.makeDomainArea(options={"ne": [nx, ny], "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
    "P0": [0.0, 0.0], "P1": [nx * 1.0, 0.0], "P2": [0.0, ny * 1.0],
    "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
for tag in sorted(mesh["Nodes"]):
    n = mesh["Nodes"][tag]
    SVL.addNode(tag=tag, ndof=n["ndof"], coords=list(map(float, n["coords"])))
for tag in sorted(mesh["Elements"]):
    el = mesh["Elements"][tag]
    SVL.addElement(tag=tag, conn=list(el["conn"]), name=el["name"], attributes=dict(el["attributes"]))
for tag in sorted(mesh["Nodes"]):
    t = tag - 1; i = t % (nx + 1); j = t // (nx + 1)
    if j == 0:
        SVL.addRestrain(tag=tag, dof=[1, 2])
etags = sorted(mesh["Elements"])
SVL.addDamping(tag=1, name="Rayleigh", attributes={"am": 4.0, "list": [e for e in etags if e % 2 == 1]})
SVL.addDamping(tag=2, name="Rayleigh", attributes={"am": 2.5, "ak": 1.5e-3, "list": [e for e in etags if e % 2 == 0]})
write_series("ricker.txt", ricker(nt, dt, 20.0, 1.0e5))
top = ny * (nx + 1) + nx // 2 + 1
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "ricker.txt", "dir": [1.0, -1.0]})
SVL.addLoad(tag=1, name="PointLoad", attributes={"type": "Concentrated", "fun": 1, "list": [top]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [1.0]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Disp.out", "ndps": 8, "resp": "disp", "list": [top]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "Newmark", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Petsc", "option": "KSPCG", "tol": 1.0e-12})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # Q4 box with a consistent mass and Rayleigh damping with ak on half the
    # elements, CentralDifference + Eigen: a non-diagonal central-difference system
    "q4_consistent_cd": COMMON + r'''
SVL.Options["dimension"] = 2
SVL.Options["massform"] = "consistent"
nx, ny, dt, nt = 6, 4, 2.5e-4, 61
SVL.addMaterial(tag=1, name="Elastic2DPlaneStrain", attributes={"E": 2.0e8, "nu": 0.25, "rho": 2000.0})
SVL.addMaterial(tag=2, name="Elastic2DPlaneStrain", attributes={"E": 3.0e8, "nu": 0.30, "rho": 2100.0})
mesh = SVL.makeDomainArea(options={"ne": [nx, ny], "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
    "P0": [0.0, 0.0], "P1": [nx * 1.0, 0.0], "P2": [0.0, ny * 1.0],
    "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
for tag in sorted(mesh["Nodes"]):
    n = mesh["Nodes"][tag]
    SVL.addNode(tag=tag, ndof=n["ndof"], coords=list(map(float, n["coords"])))
for tag in sorted(mesh["Elements"]):
    el = mesh["Elements"][tag]
    at = dict(el["attributes"])
    if tag % 4 == 0:
        at["material"] = 2
    SVL.addElement(tag=tag, conn=list(el["conn"]), name=el["name"], attributes=at)
for tag in sorted(mesh["Nodes"]):
    t = tag - 1; i = t % (nx + 1); j = t // (nx + 1)
    if j == 0:
        SVL.addRestrain(tag=tag, dof=[1, 2])
    elif i == 0 or i == nx:
        SVL.addRestrain(tag=tag, dof=1)
etags = sorted(mesh["Elements"])
SVL.addDamping(tag=1, name="Rayleigh", attributes={"am": 3.0, "list": [e for e in etags if e % 2 == 1]})
SVL.addDamping(tag=2, name="Rayleigh", attributes={"am": 1.5, "ak": 5.0e-4, "list": [e for e in etags if e % 2 == 0]})
write_series("ricker.txt", ricker(nt, dt, 60.0, 1.0e5))
top = ny * (nx + 1) + nx // 2 + 1
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "ricker.txt", "dir": [1.0, -1.0]})
SVL.addLoad(tag=1, name="PointLoad", attributes={"type": "Concentrated", "fun": 1, "list": [top]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [1.0]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Disp.out", "ndps": 8, "resp": "disp", "list": [top, top - 1]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "CentralDifference", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Eigen", "update": "OFF"})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # Q4 soil box with PML2DQuad4 layers on the sides and the bottom (setPMLDomain
    # + mergeDomain), outer PML boundary fixed, ExtendedNewmark + Eigen
    "q4_pml_extended": COMMON + r'''
SVL.Options["dimension"] = 2
SVL.Options["massform"] = "lumped"
W, H, P, dt, nt = 6.0, 4.0, 2.0, 2.0e-3, 41
SVL.addMaterial(tag=1, name="Elastic2DPlaneStrain", attributes={"E": 2.0e8, "nu": 0.25, "rho": 2000.0})
soil = SVL.makeDomainArea(options={"ne": [6, 4], "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
    "P0": [0.0, 0.0], "P1": [W, 0.0], "P2": [0.0, H],
    "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
pml = SVL.setPMLDomain({"ne": [10, 6], "ndof": 5, "class": "PML2DQUAD4", "elems": "QUAD4",
    "P0": [-P, -P], "P1": [W + P, -P], "P2": [-P, H],
    "attributes": {"material": 1, "th": 1.0, "n": 2.0, "L": P, "R": 1.0e-6, "rule": "Gauss", "np": 4}},
    [W / 2.0, H / 2.0], [W / 2.0, H / 2.0])
mesh = SVL.mergeDomain(soil, pml)
SVL.Entities["Nodes"] = mesh["Nodes"]
SVL.Entities["Elements"] = mesh["Elements"]
SVL.Entities["Constraints"] = mesh["Constraints"]        # EQUAL ties of the PML interface nodes
for tag in sorted(mesh["Nodes"]):
    x, y = mesh["Nodes"][tag]["coords"][:2]
    if abs(x + P) < 1e-9 or abs(x - W - P) < 1e-9 or abs(y + P) < 1e-9:
        SVL.addRestrain(tag=tag, dof=[1, 2])
top = [t for t in sorted(mesh["Nodes"]) if abs(mesh["Nodes"][t]["coords"][1] - H) < 1e-9 and abs(mesh["Nodes"][t]["coords"][0] - W / 2) < 1e-9][0]
write_series("ricker.txt", ricker(nt, dt, 25.0, 1.0e5))
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "ricker.txt", "dir": [0.0, -1.0]})
SVL.addLoad(tag=1, name="PointLoad", attributes={"type": "Concentrated", "fun": 1, "list": [top]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [1.0]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Disp.out", "ndps": 8, "resp": "disp", "list": [top]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "ExtendedNewmark", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Eigen", "update": "OFF"})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # The PML box with J2 (PlasticPlaneStrainJ2) top soil layers, Newmark +
    # Newton (3 iterations, the pre-processor's default convergence test)
    "q4_pml_j2_newton": COMMON + r'''
SVL.Options["dimension"] = 2
SVL.Options["massform"] = "lumped"
W, H, P, dt, nt = 6.0, 4.0, 2.0, 2.0e-3, 41
G = 2.0e8 / 2.5
K = 2.0e8 / 1.5
SVL.addMaterial(tag=1, name="Elastic2DPlaneStrain", attributes={"E": 2.0e8, "nu": 0.25, "rho": 2000.0})
SVL.addMaterial(tag=2, name="PlasticPlaneStrainJ2", attributes={"K": K, "G": G, "rho": 2000.0, "h": 0.02 * G,
                                                                 "beta": 0.5, "Sy": math.sqrt(3.0) * 15.0e3})
soil = SVL.makeDomainArea(options={"ne": [6, 4], "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
    "P0": [0.0, 0.0], "P1": [W, 0.0], "P2": [0.0, H],
    "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
for tag in soil["Elements"]:
    el = soil["Elements"][tag]
    if min(soil["Nodes"][n]["coords"][1] for n in el["conn"]) >= H - 2.0 - 1e-9:
        el["attributes"]["material"] = 2
pml = SVL.setPMLDomain({"ne": [10, 6], "ndof": 5, "class": "PML2DQUAD4", "elems": "QUAD4",
    "P0": [-P, -P], "P1": [W + P, -P], "P2": [-P, H],
    "attributes": {"material": 1, "th": 1.0, "n": 2.0, "L": P, "R": 1.0e-6, "rule": "Gauss", "np": 4}},
    [W / 2.0, H / 2.0], [W / 2.0, H / 2.0])
mesh = SVL.mergeDomain(soil, pml)
SVL.Entities["Nodes"] = mesh["Nodes"]
SVL.Entities["Elements"] = mesh["Elements"]
SVL.Entities["Constraints"] = mesh["Constraints"]
for tag in sorted(mesh["Nodes"]):
    x, y = mesh["Nodes"][tag]["coords"][:2]
    if abs(x + P) < 1e-9 or abs(x - W - P) < 1e-9 or abs(y + P) < 1e-9:
        SVL.addRestrain(tag=tag, dof=[1, 2])
top = [t for t in sorted(mesh["Nodes"]) if abs(mesh["Nodes"][t]["coords"][1] - H) < 1e-9 and abs(mesh["Nodes"][t]["coords"][0] - W / 2) < 1e-9][0]
write_series("ricker.txt", ricker(nt, dt, 25.0, 1.0e6))
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "ricker.txt", "dir": [1.0, -1.0]})
SVL.addLoad(tag=1, name="PointLoad", attributes={"type": "Concentrated", "fun": 1, "list": [top]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [1.0]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Disp.out", "ndps": 8, "resp": "disp", "list": [top]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Newton", "nstep": 3, "cnvgtol": 1.0e-12})
SVL.addIntegrator(tag=1, attributes={"name": "Newmark", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Eigen", "update": "OFF"})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # Q4 box with a fixed bottom, Rayleigh damping and a reaction recorder on
    # base nodes, CD
    "q4_reaction_cd": COMMON + r'''
SVL.Options["dimension"] = 2
SVL.Options["massform"] = "lumped"
nx, ny, dt, nt = 6, 4, 1.0e-3, 41
SVL.addMaterial(tag=1, name="Elastic2DPlaneStrain", attributes={"E": 2.0e8, "nu": 0.25, "rho": 2000.0})
mesh = SVL.makeDomainArea(options={"ne": [nx, ny], "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
    "P0": [0.0, 0.0], "P1": [nx * 1.0, 0.0], "P2": [0.0, ny * 1.0],
    "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
for tag in sorted(mesh["Nodes"]):
    n = mesh["Nodes"][tag]
    SVL.addNode(tag=tag, ndof=n["ndof"], coords=list(map(float, n["coords"])))
for tag in sorted(mesh["Elements"]):
    el = mesh["Elements"][tag]
    SVL.addElement(tag=tag, conn=list(el["conn"]), name=el["name"], attributes=dict(el["attributes"]))
base = []
for tag in sorted(mesh["Nodes"]):
    t = tag - 1; i = t % (nx + 1); j = t // (nx + 1)
    if j == 0:
        SVL.addRestrain(tag=tag, dof=[1, 2]); base.append(tag)
    elif i == 0 or i == nx:
        SVL.addRestrain(tag=tag, dof=1)
SVL.addDamping(tag=1, name="Rayleigh", attributes={"am": 3.0, "list": sorted(mesh["Elements"])})
write_series("ricker.txt", ricker(nt, dt, 25.0, 1.0e5))
top = ny * (nx + 1) + nx // 2 + 1
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "ricker.txt", "dir": [0.0, -1.0]})
SVL.addLoad(tag=1, name="PointLoad", attributes={"type": "Concentrated", "fun": 1, "list": [top]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [1.0]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Reaction.out", "ndps": 8, "resp": "reaction", "list": base[:4]})
SVL.addRecorder(tag=2, attributes={"name": "NODE", "file": "Disp.out", "ndps": 8, "resp": "disp", "list": [top]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "CentralDifference", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Eigen", "update": "OFF"})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # Q4 soil column on Lysmer dashpots (ZeroLength1D + Viscous1DLinear to fixed
    # anchor nodes at the base), periodic-free sides, CentralDifference
    "q4_lysmer_cd": COMMON + r'''
SVL.Options["dimension"] = 2
SVL.Options["massform"] = "lumped"
nx, ny, h, dt, nt = 4, 8, 0.5, 2.0e-4, 301
rho, E, nu = 2000.0, 2.0e8, 0.25
G = E / 2.0 / (1 + nu); lam = E * nu / (1 + nu) / (1 - 2 * nu)
vp, vs = math.sqrt((lam + 2 * G) / rho), math.sqrt(G / rho)
SVL.addMaterial(tag=1, name="Elastic2DPlaneStrain", attributes={"E": E, "nu": nu, "rho": rho})
SVL.addMaterial(tag=2, name="Viscous1DLinear", attributes={"eta": rho * vp * h})
SVL.addMaterial(tag=3, name="Viscous1DLinear", attributes={"eta": rho * vs * h})
mesh = SVL.makeDomainArea(options={"ne": [nx, ny], "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
    "P0": [0.0, 0.0], "P1": [nx * h, 0.0], "P2": [0.0, ny * h],
    "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
for tag in sorted(mesh["Nodes"]):
    n = mesh["Nodes"][tag]
    SVL.addNode(tag=tag, ndof=n["ndof"], coords=list(map(float, n["coords"])))
for tag in sorted(mesh["Elements"]):
    el = mesh["Elements"][tag]
    SVL.addElement(tag=tag, conn=list(el["conn"]), name=el["name"], attributes=dict(el["attributes"]))
base = [t for t in sorted(mesh["Nodes"]) if abs(mesh["Nodes"][t]["coords"][1]) < 1e-9]
ntag = max(mesh["Nodes"]) + 1
etag = max(mesh["Elements"]) + 1
for t in base:
    SVL.addNode(tag=ntag, ndof=2, coords=list(map(float, mesh["Nodes"][t]["coords"])))
    SVL.addRestrain(tag=ntag, dof=[1, 2])
    SVL.addElement(tag=etag, conn=[ntag, t], name="ZeroLength1D", attributes={"material": 3, "dir": 1})
    SVL.addElement(tag=etag + 1, conn=[ntag, t], name="ZeroLength1D", attributes={"material": 2, "dir": 2})
    ntag += 1
    etag += 2
top = [t for t in sorted(mesh["Nodes"]) if abs(mesh["Nodes"][t]["coords"][1] - ny * h) < 1e-9]
write_series("pulse.txt", ricker(nt, dt, 60.0, 2.0e4))
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "pulse.txt", "dir": [1.0, -0.5]})
SVL.addLoad(tag=1, name="PointLoad", attributes={"type": "Concentrated", "fun": 1, "list": top})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [1.0]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Base.out", "ndps": 8, "resp": "disp", "list": base[:2]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "CentralDifference", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Eigen", "update": "OFF"})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # Q4 box with a one-element domain-reduction ring; free-field motion of an
    # SV pulse in per-node files (nt nFields cond), Newmark + Eigen
    "q4_drm_newmark": COMMON + r'''
import os
SVL.Options["dimension"] = 2
SVL.Options["massform"] = "lumped"
nx, ny, h, dt, nt = 8, 6, 1.0, 1.0e-3, 41
rho, E, nu = 2000.0, 2.0e8, 0.25
G = E / 2.0 / (1 + nu)
vs = math.sqrt(G / rho)
SVL.addMaterial(tag=1, name="Elastic2DPlaneStrain", attributes={"E": E, "nu": nu, "rho": rho})
mesh = SVL.makeDomainArea(options={"ne": [nx, ny], "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
    "P0": [0.0, 0.0], "P1": [nx * h, 0.0], "P2": [0.0, ny * h],
    "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
for tag in sorted(mesh["Nodes"]):
    n = mesh["Nodes"][tag]
    SVL.addNode(tag=tag, ndof=n["ndof"], coords=list(map(float, n["coords"])))
for tag in sorted(mesh["Elements"]):
    el = mesh["Elements"][tag]
    SVL.addElement(tag=tag, conn=list(el["conn"]), name=el["name"], attributes=dict(el["attributes"]))
for tag in sorted(mesh["Nodes"]):
    x, y = mesh["Nodes"][tag]["coords"][:2]
    if abs(y) < 1e-9:
        SVL.addRestrain(tag=tag, dof=[1, 2])
    elif abs(x) < 1e-9 or abs(x - nx * h) < 1e-9:
        SVL.addRestrain(tag=tag, dof=1)
inner = lambda p: p[0] >= h - 1e-9 and p[0] <= (nx - 1) * h + 1e-9 and p[1] >= h - 1e-9
drm = []
for tag in sorted(mesh["Elements"]):
    ins = [inner(mesh["Nodes"][n]["coords"]) for n in mesh["Elements"][tag]["conn"]]
    if any(ins) and not all(ins):
        drm.append(tag)
nodes = sorted({n for e in drm for n in mesh["Elements"][e]["conn"]})
os.makedirs("drm", exist_ok=True)
for n in nodes:
    x, y = mesh["Nodes"][n]["coords"][:2]
    rows = []
    for k in range(nt):
        def g(tau):
            a = (math.pi * 20.0 * (tau - 0.06)) ** 2
            return 1e-3 * (1 - 2 * a) * math.exp(-a)
        t = k * dt - (ny * h - y) / vs
        u = g(t); v = (g(t + dt) - g(t - dt)) / (2 * dt); a = (g(t + dt) - 2 * g(t) + g(t - dt)) / dt ** 2
        rows.append("%.17g 0 %.17g 0 %.17g 0" % (u, v, a))
    with open("drm/node%d.txt" % n, "w") as f:
        f.write("%d 6 %d\n" % (nt, 0 if inner(mesh["Nodes"][n]["coords"]) else 1))
        f.write("\n".join(rows) + "\n")
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "drm/node$.txt"})
SVL.addLoad(tag=1, name="ElementLoad", attributes={"type": "GeneralWave", "fun": 1, "list": drm})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [1.0]})
top = [t for t in sorted(mesh["Nodes"]) if abs(mesh["Nodes"][t]["coords"][1] - ny * h) < 1e-9]
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Top.out", "ndps": 8, "resp": "disp", "list": top[:3]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "Newmark", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Eigen", "update": "OFF"})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # the J2 soil column with ELEMENT recorders of stress, strain, internal
    # force and strain rate (Recorder.cpp:107-166, 272-323), CentralDifference
    "q4_j2_element_cd": COMMON + r'''
SVL.Options["dimension"] = 2
SVL.Options["massform"] = "lumped"
nx, ny, h, dt, nt = 2, 6, 0.5, 2.0e-4, 61
G = 2000.0 * 200.0 ** 2; K = 2 * G * 1.3 / (3 * 0.4)
SVL.addMaterial(tag=1, name="PlasticPlaneStrainJ2", attributes={"K": K, "G": G, "rho": 2000.0, "h": 0.02 * G,
                                                                 "beta": 1.0, "Sy": math.sqrt(3.0) * 40.0e3})
mesh = SVL.makeDomainArea(options={"ne": [nx, ny], "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
    "P0": [0.0, 0.0], "P1": [nx * h, 0.0], "P2": [0.0, ny * h],
    "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
for tag in sorted(mesh["Nodes"]):
    n = mesh["Nodes"][tag]
    SVL.addNode(tag=tag, ndof=n["ndof"], coords=list(map(float, n["coords"])))
for tag in sorted(mesh["Elements"]):
    el = mesh["Elements"][tag]
    SVL.addElement(tag=tag, conn=list(el["conn"]), name=el["name"], attributes=dict(el["attributes"]))
base = [t for t in sorted(mesh["Nodes"]) if (t - 1) // (nx + 1) == 0]
for tag in base:
    SVL.addRestrain(tag=tag, dof=[1, 2])
ctag = -2
for tag in sorted(mesh["Nodes"]):
    i = (tag - 1) % (nx + 1)
    if i != nx or tag in base:
        continue
    for d in range(2):
        SVL.addConstraint(tag=ctag, name="Equal", attributes={"stag": tag, "sdof": d + 1, "mtag": [tag - nx], "mdof": [d + 1]})
        ctag -= 1
motion = [0.02 * math.sin(2 * math.pi * 8.0 * k * dt) * (1 - math.exp(-k / 10.0)) for k in range(nt)]
write_series("base.txt", motion)
for tag in base:
    SVL.addSupportMotion(tag=tag, attributes={"type": "TimeSeries", "file": "base.txt", "dof": 1})
SVL.addFunction(tag=1, name="Constant", attributes={"mag": 0.0, "dir": [0.0, -1.0]})
SVL.addLoad(tag=1, name="PointLoad", attributes={"type": "Concentrated", "fun": 1, "list": [max(mesh["Nodes"])]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [1.0]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Top.out", "ndps": 8, "resp": "disp", "list": [max(mesh["Nodes"])]})
SVL.addRecorder(tag=2, attributes={"name": "ELEMENT", "file": "Stress.out", "ndps": 10, "resp": "stress", "list": [1, 4, 12]})
SVL.addRecorder(tag=3, attributes={"name": "ELEMENT", "file": "Strain.out", "ndps": 10, "resp": "strain", "list": [2, 11]})
SVL.addRecorder(tag=4, attributes={"name": "ELEMENT", "file": "Force.out", "ndps": 10, "resp": "internalforce", "list": [1, 12]})
SVL.addRecorder(tag=5, attributes={"name": "ELEMENT", "file": "Rate.out", "ndps": 6, "resp": "strainrate", "list": [3]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "CentralDifference", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Eigen", "update": "OFF"})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # the body-loaded H8 box with ELEMENT recorders, Newmark
    "h8_element_newmark": COMMON + r'''
SVL.Options["dimension"] = 3
SVL.Options["massform"] = "lumped"
nx, ny, nz, dt, nt = 3, 3, 2, 2.0e-3, 31
SVL.addMaterial(tag=1, name="Elastic3DLinear", attributes={"E": 2.0e8, "nu": 0.3, "rho": 2000.0})
mesh = SVL.makeDomainVolume(options={"ne": [nx, ny, nz], "ndof": 3, "class": "LIN3DHEXA8", "elems": "HEXA8",
    "P0": [0.0, 0.0, 0.0], "P1": [nx * 2.0, 0.0, 0.0], "P2": [0.0, ny * 2.0, 0.0], "P3": [0.0, 0.0, nz * 2.0],
    "attributes": {"material": 1, "rule": "Gauss", "np": 8}})
for tag in sorted(mesh["Nodes"]):
    n = mesh["Nodes"][tag]
    SVL.addNode(tag=tag, ndof=n["ndof"], coords=list(map(float, n["coords"])))
for tag in sorted(mesh["Elements"]):
    el = mesh["Elements"][tag]
    SVL.addElement(tag=tag, conn=list(el["conn"]), name=el["name"], attributes=dict(el["attributes"]))
for tag in sorted(mesh["Nodes"]):
    t = tag - 1; k = t // ((nx + 1) * (ny + 1))
    if k == 0:
        SVL.addRestrain(tag=tag, dof=[1, 2, 3])
write_series("body.txt", ricker(nt, dt, 20.0, 1.0))
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "body.txt", "dir": [1.0, 0.0, 0.0]})
SVL.addLoad(tag=1, name="ElementLoad", attributes={"type": "Body", "fun": 1, "list": [8, 11]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [2.0e3]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Disp.out", "ndps": 10, "resp": "disp", "list": [40, 48]})
SVL.addRecorder(tag=2, attributes={"name": "ELEMENT", "file": "Stress.out", "ndps": 10, "resp": "stress", "list": [1, 8, 18]})
SVL.addRecorder(tag=3, attributes={"name": "ELEMENT", "file": "Force.out", "ndps": 10, "resp": "internalforce", "list": [8]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "Newmark", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Petsc", "option": "KSPCG", "tol": 1.0e-10})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
    # the merged PML box with a REACTION recorder on restrained PML nodes,
    # Newmark (PML elements add K u + C v + M a over all their dofs)
    "q4_pml_reaction_newmark": COMMON + r'''
SVL.Options["dimension"] = 2
SVL.Options["massform"] = "lumped"
W, H, P, dt, nt = 6.0, 4.0, 2.0, 2.0e-3, 41
SVL.addMaterial(tag=1, name="Elastic2DPlaneStrain", attributes={"E": 2.0e8, "nu": 0.25, "rho": 2000.0})
soil = SVL.makeDomainArea(options={"ne": [6, 4], "ndof": 2, "class": "LIN2DQUAD4", "elems": "QUAD4",
    "P0": [0.0, 0.0], "P1": [W, 0.0], "P2": [0.0, H],
    "attributes": {"material": 1, "th": 1.0, "rule": "Gauss", "np": 4}})
pml = SVL.setPMLDomain({"ne": [10, 6], "ndof": 5, "class": "PML2DQUAD4", "elems": "QUAD4",
    "P0": [-P, -P], "P1": [W + P, -P], "P2": [-P, H],
    "attributes": {"material": 1, "th": 1.0, "n": 2.0, "L": P, "R": 1.0e-6, "rule": "Gauss", "np": 4}},
    [W / 2.0, H / 2.0], [W / 2.0, H / 2.0])
mesh = SVL.mergeDomain(soil, pml)
SVL.Entities["Nodes"] = mesh["Nodes"]
SVL.Entities["Elements"] = mesh["Elements"]
SVL.Entities["Constraints"] = mesh["Constraints"]        # EQUAL ties of the PML interface nodes
fixed = []
for tag in sorted(mesh["Nodes"]):
    x, y = mesh["Nodes"][tag]["coords"][:2]
    if abs(x + P) < 1e-9 or abs(x - W - P) < 1e-9 or abs(y + P) < 1e-9:
        SVL.addRestrain(tag=tag, dof=[1, 2]); fixed.append(tag)
top = [t for t in sorted(mesh["Nodes"]) if abs(mesh["Nodes"][t]["coords"][1] - H) < 1e-9 and abs(mesh["Nodes"][t]["coords"][0] - W / 2) < 1e-9][0]
write_series("ricker.txt", ricker(nt, dt, 25.0, 1.0e5))
SVL.addFunction(tag=1, name="TimeSeries", attributes={"file": "ricker.txt", "dir": [0.0, -1.0]})
SVL.addLoad(tag=1, name="PointLoad", attributes={"type": "Concentrated", "fun": 1, "list": [top]})
SVL.addCombinationCase(tag=1, name="Fixture", attributes={"load": [1], "factor": [1.0]})
SVL.addRecorder(tag=1, attributes={"name": "NODE", "file": "Disp.out", "ndps": 8, "resp": "disp", "list": [top]})
SVL.addRecorder(tag=2, attributes={"name": "NODE", "file": "Reaction.out", "ndps": 8, "resp": "reaction", "list": fixed[:6]})
SVL.addAnalysis(tag=1, attributes={"name": "Dynamic", "nt": nt})
SVL.addAlgorithm(tag=1, attributes={"name": "Linear", "nstep": 1})
SVL.addIntegrator(tag=1, attributes={"name": "Newmark", "dt": dt})
SVL.addSolver(tag=1, attributes={"name": "Eigen", "update": "OFF"})
SVL.addSimulation(tag=1, combo=1, attributes={"analysis": 1, "algorithm": 1, "integrator": 1, "solver": 1})
SVL.CreateRunAnalysisFiles()
''',
}


def main(ref_root: str, only=None):
    pp = Path(ref_root) / "01-Pre_Process"
    scratch = HERE / ".pp_scratch"
    if scratch.exists():
        shutil.rmtree(scratch)
    stub = scratch / "stub" / "matplotlib"
    stub.mkdir(parents=True)
    (stub / "__init__.py").write_text("def use(*a, **k):\n    pass\n")
    for mod in ("pyplot.py", "pylab.py"):
        (stub / mod).write_text("def __getattr__(name):\n    return lambda *a, **k: None\n")
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([str(scratch / "stub"), str(pp)]))
    for name, script in CASES.items():
        if only and name not in only:
            continue
        work = scratch / name
        work.mkdir(parents=True)
        r = subprocess.run([sys.executable, "-c", script, name], cwd=work, env=env, capture_output=True, text=True,
                           timeout=300)
        if r.returncode != 0:
            raise SystemExit("pre-processor failed for %s:\n%s\n%s" % (name, r.stdout, r.stderr))
        out = HERE / ("partition_%s" % name)
        if out.exists():
            shutil.rmtree(out)
        (out / "Partition").mkdir(parents=True)
        for p in (work / "Partition").glob("*.json"):
            shutil.copy(p, out / "Partition" / p.name)
        for p in work.glob("*.txt"):
            shutil.copy(p, out / p.name)
        if (work / "drm").is_dir():
            shutil.copytree(work / "drm", out / "drm")
        print("wrote", out.name, sorted(x.name for x in out.rglob("*") if x.is_file()))
    shutil.rmtree(scratch)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SVL_REFERENCE_ROOT")
    if not root:
        raise SystemExit("usage: %s <SVL source tree> [case ...]  (or set SVL_REFERENCE_ROOT)" % Path(__file__).name)
    main(root, set(sys.argv[2:]) or None)
