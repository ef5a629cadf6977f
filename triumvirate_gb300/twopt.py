"""Power spectrum multipoles (mirrors ``triumvirate.twopt``
compute_powspec / compute_powspec_in_gpp_box, twopt.py:668-1280), computed
on the GPU through ``libtrvg.so``."""
from __future__ import annotations

from . import _engine
from .dataobjs import Binning
from .parameters import _as_dict, _set_ngrid_from_cutoff
from .threept import (_amalgamate_parameters, _boxsize, _has_nz, _log,
                      _log_norm, _norm_factor, _save)


def compute_powspec_in_gpp_box(catalogue_data, degree=None, binning=None,
                               sampling_params=None, paramset=None,
                               save=False, logger=None, device=None):
    """Power spectrum multipole from a periodic-box catalogue
    (twopt.py:1179-1280, twopt.cpp:609-701)."""
    paramset = _amalgamate_parameters(
        paramset=paramset, params_sampling=sampling_params,
        degrees=None if degree is None else (0, 0, degree), binning=binning,
        form='full' if paramset is None else None,
        catalogue_type='sim', statistic_type='powspec')
    if binning is None:
        binning = Binning.from_parameter_set(paramset)
    if None in paramset['boxsize'].values():
        paramset['boxsize'] = {
            ax: (catalogue_data.bounds[ax][1] - catalogue_data.bounds[ax][0])
            * paramset['expand'] for ax in ['x', 'y', 'z']}
    if None in paramset['ngrid'].values():
        pd = _as_dict(paramset)
        _set_ngrid_from_cutoff(pd)
        paramset['ngrid'] = pd['ngrid']
    catalogue_data.periodise(_boxsize(paramset))
    _log(logger, "Catalogue box has been periodised.")
    if not _has_nz(catalogue_data):
        catalogue_data.compute_mean_density(boxsize=_boxsize(paramset))
    ctx = _engine.context_for(device, catalogue_data)
    params_c = _engine.make_params(paramset, '2pt')
    cat = _engine.catalogue_arg(catalogue_data)
    norm = _norm_factor(paramset, ctx, params_c, cat.c, catalogue_data, 1.,
                        2)
    _log_norm(logger, paramset, norm)
    _log(logger, "Measuring power spectrum from a catalogue in a periodic "
         "box in the global plane-parallel approximation...")
    results = _engine.call_powspec('trvg_compute_powspec_in_gpp_box', ctx,
                                   params_c, cat.c, binning, norm)
    _log(logger, "... measured power spectrum from a catalogue in a "
         "periodic box in the global plane-parallel approximation.")
    if save:
        path = _save(results, paramset, save, ctx, params_c, cat.c,
                     catalogue_data, 1., 2, catalogue_data)
        _log(logger, "Measurements saved to %s.", path)
    return results


def compute_powspec(catalogue_data, catalogue_rand, los_data=None,
                    los_rand=None, degree=None, binning=None,
                    sampling_params=None, paramset=None, save=False,
                    logger=None, device=None):
    """Power spectrum multipole from survey-type catalogues
    (twopt.py:668-880, twopt.cpp:388-496)."""
    paramset = _amalgamate_parameters(
        paramset=paramset, params_sampling=sampling_params,
        degrees=None if degree is None else (0, 0, degree), binning=binning,
        form='full' if paramset is None else None,
        catalogue_type='survey', statistic_type='powspec')
    if binning is None:
        binning = Binning.from_parameter_set(paramset)
    if los_data is None:
        los_data = catalogue_data.compute_los()
    if los_rand is None:
        los_rand = catalogue_rand.compute_los()
    if None in paramset['boxsize'].values():
        paramset['boxsize'] = {
            ax: (catalogue_rand.bounds[ax][1] - catalogue_rand.bounds[ax][0])
            * paramset['expand'] for ax in ['x', 'y', 'z']}
    if None in paramset['ngrid'].values():
        pd = _as_dict(paramset)
        _set_ngrid_from_cutoff(pd)
        paramset['ngrid'] = pd['ngrid']
    if paramset['alignment'] == 'centre':
        catalogue_data.centre(_boxsize(paramset), catalogue_ref=catalogue_rand)
    elif paramset['alignment'] == 'pad':
        if paramset['padscale'] == 'box':
            kw = {'boxsize_pad': paramset['padfactor']}
        else:
            kw = {'ngrid': [paramset['ngrid'][ax] for ax in 'xyz'],
                  'ngrid_pad': paramset['padfactor']}
        catalogue_data.pad(_boxsize(paramset), catalogue_ref=catalogue_rand,
                           **kw)
    _log(logger, "Catalogues have been aligned.")
    ctx = _engine.context_for(device, catalogue_data, catalogue_rand)
    params_c = _engine.make_params(paramset, '2pt')
    alpha = catalogue_data.wstotal / catalogue_rand.wstotal
    _log(logger, "Alpha contrast: %.6e.", alpha)
    dcat = _engine.catalogue_arg(catalogue_data, los_data, with_los=True)
    rcat = _engine.catalogue_arg(catalogue_rand, los_rand, with_los=True)
    norm = _norm_factor(paramset, ctx, params_c, rcat.c, catalogue_rand,
                        alpha, 2)
    _log_norm(logger, paramset, norm)
    _log(logger, "Measuring power spectrum from paired survey-type "
         "catalogues in the local plane-parallel approximation...")
    results = _engine.call_powspec('trvg_compute_powspec', ctx, params_c,
                                   dcat.c, binning, norm, rand_c=rcat.c,
                                   alpha=alpha)
    _log(logger, "... measured power spectrum from paired survey-type "
         "catalogues in the local plane-parallel approximation.")
    if save:
        path = _save(results, paramset, save, ctx, params_c, rcat.c,
                     catalogue_rand, alpha, 2, catalogue_data, catalogue_rand)
        _log(logger, "Measurements saved to %s.", path)
    return results
