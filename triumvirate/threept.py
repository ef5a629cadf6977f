"""``triumvirate.threept`` (threept.py of the reference) on the GPU."""
from triumvirate_gb300.threept import (  # noqa: F401
    compute_3pcf, compute_3pcf_in_gpp_box, compute_3pcf_window,
    compute_bispec, compute_bispec_in_gpp_box,
    compute_bispec_in_gpp_box_batch)
