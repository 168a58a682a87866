"""The oracle still reproduces its frozen regression vectors (tests/golden)."""
from pathlib import Path

import numpy as np

import sys
sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import make_golden as MG  # noqa: E402

GOLD = Path(__file__).resolve().parent / "golden"


def _cmp(got, ref, tol):
    for k in ref.files:
        a, b = np.asarray(got[k], dtype=float), ref[k].astype(float)
        scale = max(np.abs(b).max(), 1e-300)
        assert np.abs(a - b).max() / scale < tol, k


def test_cylinder_direct_1step():
    _cmp(MG.cylinder_case(1), np.load(GOLD / "cylinder64x32_direct_1step.npz"), 1e-11)


def test_cylinder_direct_10steps():
    _cmp(MG.cylinder_case(10), np.load(GOLD / "cylinder64x32_direct_10steps.npz"), 1e-9)


def test_plate_gmres_3steps():
    got = MG.plate_case(3)
    ref = np.load(GOLD / "plate64x32_gmres_3steps.npz")
    assert np.array_equal(got["fsi"], ref["fsi"])
    assert np.abs(got["theta"] - ref["theta"]).max() < 1e-8 * np.abs(ref["theta"]).max()
    for k in ("omega0", "f", "xb"):
        assert np.abs(got[k] - ref[k]).max() < 1e-6 * np.abs(ref[k]).max(), k
