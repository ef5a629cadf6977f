"""``triumvirate.transforms`` (transforms.py of the reference)."""
from triumvirate_gb300.transforms import (  # noqa: F401
    DoubleSphericalBesselTransform, SphericalBesselTransform, resample_lglin,
    resample_lin)
