"""``triumvirate.parameters`` (parameters.pyx of the reference)."""
from triumvirate_gb300.parameters import (  # noqa: F401
    InvalidParameterError, ParameterSet, fetch_paramset_template)
