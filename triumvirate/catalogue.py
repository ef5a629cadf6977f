"""``triumvirate.catalogue`` (catalogue.py of the reference)."""
from triumvirate_gb300.catalogue import (  # noqa: F401
    DeviceCatalogue, ParticleCatalogue)
