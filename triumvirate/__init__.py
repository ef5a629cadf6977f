"""The reference's import path (``import triumvirate``) served by the GB300
library: each submodule forwards the public names of the matching
``triumvirate_gb300`` module, so code written against MikeSWang/Triumvirate
(``from triumvirate.threept import compute_bispec`` and so on) runs on the
GPU unchanged.  Every estimator takes one more keyword, ``device``, and the
parameter set one more key, ``precision`` ('fp64' or 'fp32mixed')."""
from triumvirate_gb300 import __all__ as _gb300_all  # noqa: F401

__all__ = ['catalogue', 'dataobjs', 'logger', 'parameters', 'threept',
           'transforms', 'twopt']
