"""``triumvirate.dataobjs`` (dataobjs.pyx of the reference)."""
from triumvirate_gb300.dataobjs import Binning  # noqa: F401
