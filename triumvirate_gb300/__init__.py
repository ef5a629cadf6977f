"""GB300-native mesh-based clustering estimators with Triumvirate's API.

Bispectrum / 3PCF / power-spectrum multipoles from particle catalogues,
computed by hand-written sm_103a CUDA kernels and cuFFT behind a C ABI
(``include/trvg.h``, ``libtrvg.so``).  The Python surface mirrors the
reference package ``triumvirate``:

* ``threept.compute_bispec``, ``compute_bispec_in_gpp_box``,
  ``compute_3pcf``, ``compute_3pcf_in_gpp_box``, ``compute_3pcf_window``;
* ``twopt.compute_powspec``, ``compute_powspec_in_gpp_box``;
* ``catalogue.ParticleCatalogue``, ``parameters.ParameterSet``,
  ``parameters.fetch_paramset_template``, ``dataobjs.Binning``;
* ``transforms`` (spherical-Bessel / FFTLog transforms), ``io``
  (measurement files).

Beyond it: ``catalogue.DeviceCatalogue`` (catalogues read into and
prepared in GPU memory), ``threept.compute_bispec_in_gpp_box_batch``
(mocks of uneven sizes in one call, replayed from a captured CUDA graph),
``adjoint`` (gradients of the bispectrum behind ``torch.autograd``) and
``replicas`` (independent estimates spread over GPUs).
"""
__version__ = "0.1.0"

__all__ = ["catalogue", "dataobjs", "parameters", "threept", "twopt"]
