"""Extracts the reference validation data the oracle pins use into
tests/golden/pins/: the load series and the OpenSees displacement histories
shipped with the reference's validation cases F02 (lin2DQuad4, elastic,
Newmark), F03 (lin2DQuad4, PlasticPlaneStrainJ2, Newton) and J02
(lin3DHexa8, elastic, Newmark), 03-Validations/01-Debugging/<case>.zip.

    python tests/golden/make_pin_fixtures.py <SVL source tree>

(or set SVL_REFERENCE_ROOT).  The files are copied byte for byte.
"""
import os
import sys
import zipfile
from pathlib import Path

HERE = Path(__file__).resolve().parent / "pins"
CASES = {
    "F02-DY_Lin_2DPointLoad_ElasticPStrain_Quad4": ("StressLoad.txt", "OpenSees/displacement.out"),
    "F03-DY_Lin_2DPointLoad_J2PStrain_Quad4": ("ricker.in", "OpenSees/displacement.out"),
    "J02-DY_Lin_3DPointLoad_Elastic_Hexa8": ("StressLoad.txt", "OpenSees/displacement.out"),
}


def main(root):
    HERE.mkdir(exist_ok=True)
    for case, members in CASES.items():
        with zipfile.ZipFile(Path(root) / "03-Validations" / "01-Debugging" / (case + ".zip")) as z:
            for mem in members:
                out = HERE / (case.split("-")[0] + "_" + mem.replace("/", "_"))
                out.write_bytes(z.read(case + "/" + mem))
                print("wrote", out.name)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SVL_REFERENCE_ROOT")
    if not root:
        raise SystemExit("usage: make_pin_fixtures.py <SVL source tree>  (or set SVL_REFERENCE_ROOT)")
    main(root)
