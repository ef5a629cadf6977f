"""``triumvirate.twopt`` (twopt.py of the reference): the power-spectrum
estimators, on the GPU."""
from triumvirate_gb300.twopt import (  # noqa: F401
    compute_powspec, compute_powspec_in_gpp_box)
