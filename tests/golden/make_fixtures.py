"""Copy the reference's golden measurement vectors into this folder.

The reference Triumvirate (MikeSWang/Triumvirate) ships regression goldens
for its estimators under ``tests/test_input/stats/`` and the three-particle
data catalogue under ``tests/test_input/ctlgs/``; they were produced by the
reference's own Python API (``deploy/test/gen_test_dataset.py``).  This
script copies the ones on the accelerated path verbatim, so that the tests
here can run where the reference tree is absent.

The 30 000-particle random catalogue (``test_rand_catalogue.txt``) is not
copied: it is exactly ``numpy.random.default_rng(seed=42).uniform(-500.,
500., size=(3, 30000))`` with ``nz = 3e-9`` (reference
``tests/conftest.py:173-195``); ``tests/conftest.py`` regenerates it and
``tests/test_oracle.py`` checks the regeneration against the reference
file whenever the reference tree is present.

Usage::

    python tests/golden/make_fixtures.py [REFERENCE_ROOT]
"""
import os
import shutil
import sys
from pathlib import Path

FILES = [
    "stats/bk000_diag_gpp.txt", "stats/bk000_row0_gpp.txt",
    "stats/bk202_diag_gpp.txt",
    "stats/bk000_diag_lpp.txt", "stats/bk000_row0_lpp.txt",
    "stats/bk202_diag_lpp.txt",
    "stats/zeta000_diag_gpp.txt", "stats/zeta000_row0_gpp.txt",
    "stats/zeta202_diag_gpp.txt",
    "stats/zeta000_diag_lpp.txt", "stats/zeta000_row0_lpp.txt",
    "stats/zeta202_diag_lpp.txt",
    "stats/zetaw000_diag.txt", "stats/zetaw000_row0.txt",
    "stats/zetaw202_diag.txt",
    "stats/pk0_gpp.txt", "stats/pk2_gpp.txt",
    "stats/pk0_lpp.txt", "stats/pk2_lpp.txt",
    "ctlgs/test_data_catalogue.txt",
    "params/test_params.yml",
]


def main(ref_root=None):
    ref_root = ref_root or os.environ.get("TRIUMVIRATE_REFERENCE")
    if not ref_root:
        sys.exit("usage: python %s REFERENCE_ROOT "
                 "(or set TRIUMVIRATE_REFERENCE to the reference checkout)"
                 % Path(__file__).name)
    src = Path(ref_root) / "tests" / "test_input"
    dst = Path(__file__).resolve().parent
    for rel in FILES:
        out = dst / Path(rel).name
        shutil.copyfile(src / rel, out)
        print(f"copied {rel} -> {out.name}")


if __name__ == "__main__":
    main(*sys.argv[1:])
