"""Power spectrum multipoles (mirrors ``triumvirate.twopt``
compute_powspec / compute_powspec_in_gpp_box, twopt.py:668-1280), computed
on the GPU through ``libtrvg.so``."""
from __future__ import annotations

import numpy as np

from . import _engine, _lib
from .dataobjs import Binning
from .parameters import _as_dict, _set_ngrid_from_cutoff
from .threept import _amalgamate_parameters, _boxsize, _norm_factor, _save


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
    if not catalogue_data['nz'].any():
        catalogue_data.compute_mean_density(boxsize=_boxsize(paramset))
    ctx = _lib.default_context(device)
    params_c = _engine.make_params(paramset, '2pt')
    x, y, z, w = catalogue_data._columns()
    cat = _engine.HostCatalogue(x, y, z, w)
    norm = _norm_factor(paramset, ctx, params_c, cat.c, catalogue_data['nz'],
                        catalogue_data['ws'], catalogue_data['wc'], 1., 2)
    results = _engine.call_powspec('trvg_compute_powspec_in_gpp_box', ctx,
                                   params_c, cat.c, binning, norm)
    if save:
        _save(results, paramset, save, ctx, params_c, cat.c,
              catalogue_data['nz'], catalogue_data['ws'], catalogue_data['wc'],
              1., 2, catalogue_data)
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
    ctx = _lib.default_context(device)
    params_c = _engine.make_params(paramset, '2pt')
    alpha = catalogue_data.wstotal / catalogue_rand.wstotal
    xd, yd, zd, wd = catalogue_data._columns()
    xr, yr, zr, wr = catalogue_rand._columns()
    dcat = _engine.HostCatalogue(xd, yd, zd, wd, np.asarray(los_data))
    rcat = _engine.HostCatalogue(xr, yr, zr, wr, np.asarray(los_rand))
    norm = _norm_factor(paramset, ctx, params_c, rcat.c, catalogue_rand['nz'],
                        catalogue_rand['ws'], catalogue_rand['wc'], alpha, 2)
    results = _engine.call_powspec('trvg_compute_powspec', ctx, params_c,
                                   dcat.c, binning, norm, rand_c=rcat.c,
                                   alpha=alpha)
    if save:
        _save(results, paramset, save, ctx, params_c, rcat.c,
              catalogue_rand['nz'], catalogue_rand['ws'], catalogue_rand['wc'],
              alpha, 2, catalogue_data, catalogue_rand)
    return results
