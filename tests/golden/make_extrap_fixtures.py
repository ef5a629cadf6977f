"""Golden vectors of the oscillatory log-linear extrapolation.

Runs the reference's own ``extrap_loglin_oscil`` (pure numpy, in
``src/triumvirate/_arrayops.py`` of MikeSWang/Triumvirate) on the seeded
inputs of ``inputs()`` and writes ``extrap_loglin_oscil.npz`` beside this
script, so that ``tests/test_fftlog.py`` can compare the restatement in
``triumvirate_gb300/_arrayops.py`` where the reference tree is absent.

Usage::

    python tests/golden/make_extrap_fixtures.py [REFERENCE_ROOT]
"""
import os
import importlib.util
import sys
import warnings
from pathlib import Path

import numpy as np


def inputs():
    """Arrays covering the branches: oscillating tails, monotonic decay,
    tails growing outwards (constant padding), sign changes, zeros."""
    x = np.logspace(-3, 1, 64)
    rng = np.random.default_rng(12)
    cases = {
        "damped_oscillation": np.sin(5 * x) / x ** 2,
        "power_law": x ** -1.5,
        "growing_tails": x ** 2 + 1. / x,
        "bump": np.exp(-np.log(x) ** 2),
        "sign_change": np.cos(x) * np.exp(-x / 4.),
        "noisy_decay": x ** -1 * (1. + 0.3 * rng.standard_normal(64)),
        "with_zero": np.where(np.arange(64) == 40, 0., np.sinc(x)),
        "short": np.array([1., 2., 3., 2.5, 1., 0.5, 0.2, 0.1]),
    }
    return cases


def main(ref_root=None):
    ref_root = ref_root or os.environ.get("TRIUMVIRATE_REFERENCE")
    if not ref_root:
        sys.exit("usage: python %s REFERENCE_ROOT "
                 "(or set TRIUMVIRATE_REFERENCE to the reference checkout)"
                 % Path(__file__).name)
    path = Path(ref_root) / "src" / "triumvirate" / "_arrayops.py"
    spec = importlib.util.spec_from_file_location("ref_arrayops", path)
    ref = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ref)
    out = {}
    for name, a in inputs().items():
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            out[f"{name}__in"] = a
            out[f"{name}__out"] = ref.extrap_loglin_oscil(a, 16)
    dst = Path(__file__).resolve().parent / "extrap_loglin_oscil.npz"
    np.savez(dst, **out)
    print(f"wrote {dst.name} ({len(out) // 2} cases)")


if __name__ == "__main__":
    main(*sys.argv[1:])
