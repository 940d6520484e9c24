"""Golden values for the engines' host analysis helpers getBeamWidth and
getOverlap (PtyLab/Engines/BaseEngine.py:744-818).

Test infrastructure only: calls the REFERENCE's own methods on a small
reconstruction (two probe modes, three wavelengths, positions of a Fermat
scan) and records their outputs.

    python tests/golden/make_analysis_golden.py --reference <path of a PtyLab.py checkout>

Output: ``tests/golden/analysis_golden.npz``.
"""

from __future__ import annotations

import argparse
import importlib
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))


def inputs():
    rng = np.random.default_rng(5)
    Np, dxp = 48, 2e-6
    x = np.linspace(-Np / 2, Np / 2, Np) * dxp
    Xp, Yp = np.meshgrid(x, x)
    g = np.exp(-((Xp - 3e-6) ** 2 + (Yp + 2e-6) ** 2) / (2 * (12e-6) ** 2))
    probe = (g[None, None, None, None] * (1 + 0.1 * rng.standard_normal((3, 1, 2, 1, Np, Np)))).astype(np.complex64)
    positions = np.round(rng.random((10, 2)) * 30).astype(int)
    return dict(probe=probe, Xp=Xp, Yp=Yp, positions=positions, dxp=dxp, Np=Np)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    args = ap.parse_args()
    from refload import load_reference

    load_reference(args.reference)
    be = importlib.import_module("PtyLab.Engines.BaseEngine")
    inp = inputs()
    rec = types.SimpleNamespace(**inp)
    eng = types.SimpleNamespace(reconstruction=rec)
    by, bx = be.BaseEngine.getBeamWidth(eng)
    out = {"beamWidthY": np.asarray(by), "beamWidthX": np.asarray(bx)}
    eng.getBeamWidth = lambda: be.BaseEngine.getBeamWidth(eng)
    for a, b in ((0, 3), (2, 7), (5, 5)):
        be.BaseEngine.getOverlap(eng, a, b)
        out[f"linear_{a}_{b}"] = np.asarray(rec.linearOverlap)
        out[f"area_{a}_{b}"] = np.asarray(rec.areaOverlap)
    np.savez(HERE / "analysis_golden.npz", **{f"in_{k}": v for k, v in inp.items()}, **out)
    print("wrote", HERE / "analysis_golden.npz")


if __name__ == "__main__":
    main()
