"""Three-point clustering statistics (mirrors ``triumvirate.threept``,
threept.py:1-1723): bispectrum and 3PCF from periodic-box ('sim') and
survey-type catalogues, computed on the GPU through ``libtrvg.so``."""
from __future__ import annotations

import warnings

import numpy as np

from . import _engine, _lib, io
from .catalogue import DeviceCatalogue
from .dataobjs import Binning
from .parameters import (ParameterSet, _as_dict,
                         _modify_measurement_parameters,
                         _modify_sampling_parameters, _set_ngrid_from_cutoff,
                         fetch_paramset_template)


def _amalgamate_parameters(paramset=None, params_sampling=None, degrees=None,
                           wa_orders=None, binning=None, form=None,
                           idx_bin=None, **type_kwargs):
    """Parameter set with sampling / measurement overrides
    (threept.py:53-172)."""
    if paramset is None and params_sampling is None:
        raise ValueError(
            "Either `paramset` or `sampling_params` must be provided.")
    if paramset is None and None in [degrees, binning, form]:
        raise ValueError("`degrees`, `binning` and `form` must be provided "
                         "when `paramset` is None.")
    if paramset is None and form in ['row', 'off-diag'] and idx_bin is None:
        raise ValueError("`idx_bin` must be provided when `paramset` is None "
                         "and `form` is 'row' or 'off-diag'.")
    if paramset is None:
        pdict, defaults = fetch_paramset_template('dict', ret_defaults=True)
    else:
        pdict, defaults = _as_dict(paramset), None
    if params_sampling is not None:
        pdict, defaults = _modify_sampling_parameters(
            pdict, params_sampling, params_default=defaults,
            ret_defaults=True)
    measure = {}
    if degrees is not None:
        ell1, ell2, ELL = degrees
        measure.update({'ell1': int(ell1), 'ell2': int(ell2),
                        'ELL': int(ELL)})
    if wa_orders is not None:
        i_wa, j_wa = wa_orders
        measure.update({'i_wa': int(i_wa), 'j_wa': int(j_wa)})
    if binning is not None:
        measure.update({'bin_min': binning.bin_min,
                        'bin_max': binning.bin_max,
                        'num_bins': binning.num_bins})
    if form is not None:
        measure['form'] = form
    if idx_bin is not None:
        measure['idx_bin'] = idx_bin
    pdict, defaults = _modify_measurement_parameters(
        pdict, measure, params_default=defaults, ret_defaults=True)
    pdict.update(type_kwargs)
    if defaults:
        warnings.warn("The following parameter default values are "
                      f"unchanged: {defaults}. Not all parameters are "
                      "necessarily used.", stacklevel=3)
    return ParameterSet(param_dict=pdict)


def _boxsize(paramset):
    return [float(paramset['boxsize'][ax]) for ax in ['x', 'y', 'z']]


def _log(logger, msg, *args):
    """Progress message at the reference's 'stat' level where the logger
    has one (the library's own logger, logger.py), else at INFO
    (threept.py:490-738 log the same stages)."""
    if logger is None:
        return
    fn = getattr(logger, 'stat', None) or logger.info
    fn(msg, *args)


_STAT_NAMES = {'bispec': 'bispectrum', '3pcf': 'three-point correlation '
               'function', 'powspec': 'power spectrum'}


def _log_norm(logger, paramset, norm):
    _log(logger, "Normalisation factor: %.6e (%s; used).", norm,
         paramset['norm_convention'])


def _has_nz(catalogue):
    """Whether any particle has a nonzero 'nz' (summed on the device for a
    DeviceCatalogue)."""
    if hasattr(catalogue, '_has_nz'):
        return catalogue._has_nz()
    return bool(np.asarray(catalogue['nz']).any())


def _norm_particle(catalogue, alpha, order, strict=True):
    """1 / (alpha sum ws nz^(order-1) wc^order) (threept.cpp:96-136,
    twopt.cpp:56-99)."""
    if hasattr(catalogue, '_norm_sum'):
        norm = catalogue._norm_sum(order)
    else:
        nz, ws, wc = (np.asarray(catalogue[k]) for k in ('nz', 'ws', 'wc'))
        norm = float(np.sum(ws * nz ** 2 * wc ** 3) if order == 3
                     else np.sum(ws * nz * wc ** 2))
    if norm == 0.:
        if not strict:
            return float('inf')
        raise _lib.InvalidDataError(
            "Particle 'nz' values appear to be all zeros. Check the "
            "input catalogue contains valid 'nz' field.")
    return 1. / (alpha * norm)


def _norm_mesh(ctx, params_c, cat_c, alpha, order):
    """Grid-based normalisation (threept.cpp:138-149, twopt.cpp:101-130)."""
    return _engine.grid_powlaw_norm(ctx, params_c, cat_c, order) \
        / alpha ** order


def _norm_factor(paramset, ctx, params_c, cat_c, catalogue, alpha, order):
    """Particle / mesh normalisation of the chosen convention."""
    conv = paramset['norm_convention']
    if conv == 'none':
        return 1.
    if conv == 'particle':
        return _norm_particle(catalogue, alpha, order)
    if conv == 'mesh':
        return _norm_mesh(ctx, params_c, cat_c, alpha, order)
    raise ValueError(f"Unsupported normalisation convention: {conv}.")


def _save(results, paramset, save, ctx, params_c, cat_c, catalogue, alpha,
          order, catalogue_data, catalogue_rand=None):
    """Write the measurements with the library's header: catalogue
    attributes, sampling parameters and every normalisation alternative
    (threept.py:707-735, twopt.py:633-663)."""
    part = _norm_particle(catalogue, alpha, order, strict=False)
    mesh = _norm_mesh(ctx, params_c, cat_c, alpha, order)
    header = "\n".join([
        catalogue_data.write_attrs_as_header(catalogue_ref=catalogue_rand),
        io.measurement_header(paramset, part, mesh, 0.)])
    return io.save_measurements(results, paramset, save, header)


def _compute_3pt_stats_sim_like(kind, catalogue_data, paramset=None,
                                params_sampling=None, degrees=None,
                                binning=None, form=None, idx_bin=None,
                                save=False, logger=None, device=None):
    """Periodic-box three-point statistics (threept.py:1312-1621)."""
    stat = 'bispec' if kind == 'bispec' else '3pcf'
    paramset = _amalgamate_parameters(
        paramset=paramset, params_sampling=params_sampling, degrees=degrees,
        binning=binning, form=form, idx_bin=idx_bin,
        catalogue_type='sim', statistic_type=stat)
    _log(logger, "Parameter set have been initialised.")
    if binning is None:
        binning = Binning.from_parameter_set(paramset)
    _log(logger, "Binning has been initialised.")
    if None in paramset['boxsize'].values():
        paramset['boxsize'] = {
            ax: (catalogue_data.bounds[ax][1] - catalogue_data.bounds[ax][0])
            * paramset['expand'] for ax in ['x', 'y', 'z']}
        _log(logger, "Box size is set to [%.3f, %.3f, %.3f].",
             *_boxsize(paramset))
    if None in paramset['ngrid'].values():
        pd = _as_dict(paramset)
        _set_ngrid_from_cutoff(pd)
        paramset['ngrid'] = pd['ngrid']
    catalogue_data.periodise(_boxsize(paramset))
    _log(logger, "Catalogue box has been periodised.")
    if not _has_nz(catalogue_data):
        catalogue_data.compute_mean_density(boxsize=_boxsize(paramset))

    ctx = _engine.context_for(device, catalogue_data)
    params_c = _engine.make_params(paramset, '3pt')
    cat = _engine.catalogue_arg(catalogue_data)
    norm = _norm_factor(paramset, ctx, params_c, cat.c, catalogue_data, 1.,
                        3)
    _log_norm(logger, paramset, norm)
    fn = ('trvg_compute_bispec_in_gpp_box' if kind == 'bispec'
          else 'trvg_compute_3pcf_in_gpp_box')
    _log(logger, "Measuring %s from a catalogue in a periodic box in the "
         "global plane-parallel approximation...", _STAT_NAMES[stat])
    results = _engine.call_threept(
        fn, ctx, params_c, cat.c, binning, norm, kind,
        shape=paramset['shape'], idx_bin=paramset.get('idx_bin') or 0)
    _log(logger, "... measured %s from a catalogue in a periodic box in "
         "the global plane-parallel approximation.", _STAT_NAMES[stat])
    if save:
        path = _save(results, paramset, save, ctx, params_c, cat.c,
                     catalogue_data, 1., 3, catalogue_data)
        _log(logger, "Measurements saved to %s.", path)
    return results


def _compute_3pt_stats_survey_like(kind, catalogue_data, catalogue_rand,
                                   los_data=None, los_rand=None,
                                   paramset=None, params_sampling=None,
                                   degrees=None, binning=None, form=None,
                                   idx_bin=None, save=False, logger=None,
                                   device=None):
    """Survey-type three-point statistics (threept.py:384-740)."""
    stat = 'bispec' if kind == 'bispec' else '3pcf'
    paramset = _amalgamate_parameters(
        paramset=paramset, params_sampling=params_sampling, degrees=degrees,
        binning=binning, form=form, idx_bin=idx_bin,
        catalogue_type='survey', statistic_type=stat)
    _log(logger, "Parameter set have been initialised.")
    if binning is None:
        binning = Binning.from_parameter_set(paramset)
    _log(logger, "Binning has been initialised.")
    if los_data is None:
        los_data = catalogue_data.compute_los()
    if los_rand is None:
        los_rand = catalogue_rand.compute_los()
    _log(logger, "Lines of sight have been initialised.")
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
    if paramset['alignment'] == 'pad':
        if paramset['padscale'] == 'box':
            kw = {'boxsize_pad': paramset['padfactor']}
        else:
            kw = {'ngrid': [paramset['ngrid'][ax] for ax in 'xyz'],
                  'ngrid_pad': paramset['padfactor']}
        catalogue_data.pad(_boxsize(paramset), catalogue_ref=catalogue_rand,
                           **kw)
    _log(logger, "Catalogues have been aligned.")
    ctx = _engine.context_for(device, catalogue_data, catalogue_rand)
    params_c = _engine.make_params(paramset, '3pt')
    alpha = catalogue_data.wstotal / catalogue_rand.wstotal
    _log(logger, "Alpha contrast: %.6e.", alpha)
    dcat = _engine.catalogue_arg(catalogue_data, los_data, with_los=True)
    rcat = _engine.catalogue_arg(catalogue_rand, los_rand, with_los=True)
    norm = _norm_factor(paramset, ctx, params_c, rcat.c, catalogue_rand,
                        alpha, 3)
    _log_norm(logger, paramset, norm)
    fn = 'trvg_compute_bispec' if kind == 'bispec' else 'trvg_compute_3pcf'
    _log(logger, "Measuring %s from paired survey-type catalogues in the "
         "local plane-parallel approximation...", _STAT_NAMES[stat])
    results = _engine.call_threept(
        fn, ctx, params_c, dcat.c, binning, norm, kind, rand_c=rcat.c,
        alpha=alpha, shape=paramset['shape'],
        idx_bin=paramset.get('idx_bin') or 0)
    _log(logger, "... measured %s from paired survey-type catalogues in "
         "the local plane-parallel approximation.", _STAT_NAMES[stat])
    if save:
        path = _save(results, paramset, save, ctx, params_c, rcat.c,
                     catalogue_rand, alpha, 3, catalogue_data, catalogue_rand)
        _log(logger, "Measurements saved to %s.", path)
    return results


def compute_bispec(catalogue_data, catalogue_rand, los_data=None,
                   los_rand=None, degrees=None, binning=None, form=None,
                   idx_bin=None, sampling_params=None, paramset=None,
                   save=False, logger=None, device=None):
    """Bispectrum from survey-type catalogues in the local plane-parallel
    approximation (threept.py:743-865)."""
    return _compute_3pt_stats_survey_like(
        'bispec', catalogue_data, catalogue_rand, los_data=los_data,
        los_rand=los_rand, paramset=paramset, params_sampling=sampling_params,
        degrees=degrees, binning=binning, form=form, idx_bin=idx_bin,
        save=save, logger=logger, device=device)


def compute_3pcf(catalogue_data, catalogue_rand, los_data=None,
                 los_rand=None, degrees=None, binning=None, form=None,
                 idx_bin=None, sampling_params=None, paramset=None,
                 save=False, logger=None, device=None):
    """3PCF from survey-type catalogues (threept.py:868-990)."""
    return _compute_3pt_stats_survey_like(
        '3pcf', catalogue_data, catalogue_rand, los_data=los_data,
        los_rand=los_rand, paramset=paramset, params_sampling=sampling_params,
        degrees=degrees, binning=binning, form=form, idx_bin=idx_bin,
        save=save, logger=logger, device=device)


def compute_3pcf_window(catalogue_rand, los_rand=None, degrees=None,
                        wa_orders=None, binning=None, form=None,
                        idx_bin=None, sampling_params=None, paramset=None,
                        save=False, logger=None, device=None):
    """3PCF window from a random catalogue, with wide-angle corrections of
    orders `wa_orders` (i_wa, j_wa) when given (threept.py:1832-2080).

    The random field alone, scaled by alpha = 1, takes the place of the
    data-minus-randoms field of :func:`compute_3pcf`; the normalisation is
    the randoms' own (alpha = 1).  Returns the keys of
    :func:`compute_3pcf` ('r1_bin', 'r1_eff', 'npairs_1', 'r2_*',
    'zeta_raw', 'zeta_shot')."""
    wide_angle = wa_orders is not None
    paramset = _amalgamate_parameters(
        paramset=paramset, params_sampling=sampling_params, degrees=degrees,
        wa_orders=wa_orders, binning=binning, form=form, idx_bin=idx_bin,
        catalogue_type='random', statistic_type='3pcf-win')
    _log(logger, "Parameter set have been initialised.")
    if binning is None:
        binning = Binning.from_parameter_set(paramset)
    _log(logger, "Binning has been initialised.")
    if los_rand is None:
        los_rand = catalogue_rand.compute_los()
    _log(logger, "Lines of sight have been initialised.")
    catalogue_rand.centre(_boxsize(paramset))
    catalogue_rand.periodise(_boxsize(paramset))
    _log(logger, "Catalogue box has been periodised.")
    ctx = _engine.context_for(device, catalogue_rand)
    params_c = _engine.make_params(paramset, '3pt')
    rcat = _engine.catalogue_arg(catalogue_rand, los_rand, with_los=True)
    norm = _norm_factor(paramset, ctx, params_c, rcat.c, catalogue_rand, 1.,
                        3)
    _log_norm(logger, paramset, norm)
    _log(logger, "Measuring three-point correlation function window from "
         "a random catalogue...")
    results = _engine.call_3pcf_window(
        ctx, params_c, rcat.c, binning, norm, 1., wide_angle,
        shape=paramset['shape'], idx_bin=paramset.get('idx_bin') or 0)
    _log(logger, "... measured three-point correlation function window "
         "from a random catalogue.")
    if save:
        path = _save(results, paramset, save, ctx, params_c, rcat.c,
                     catalogue_rand, 1., 3, catalogue_rand)
        _log(logger, "Measurements saved to %s.", path)
    return results


def compute_bispec_in_gpp_box(catalogue_data, degrees=None, binning=None,
                              form=None, idx_bin=None, sampling_params=None,
                              paramset=None, save=False, logger=None,
                              device=None):
    """Bispectrum from a periodic-box catalogue in the global plane-parallel
    approximation (threept.py:1624-1723)."""
    return _compute_3pt_stats_sim_like(
        'bispec', catalogue_data, paramset=paramset,
        params_sampling=sampling_params, degrees=degrees, binning=binning,
        form=form, idx_bin=idx_bin, save=save, logger=logger, device=device)


def compute_bispec_in_gpp_box_batch(catalogues, degrees=None, binning=None,
                                    form=None, idx_bin=None,
                                    sampling_params=None, paramset=None,
                                    device=None):
    """Bispectra of several periodic-box catalogues (e.g. mocks of uneven
    sizes) in one library call; returns one result dictionary per
    catalogue, each equal to that of `compute_bispec_in_gpp_box`.  The
    library has no batched counterpart: it is called once per catalogue."""
    if len(catalogues) == 0:
        return []
    paramset = _amalgamate_parameters(
        paramset=paramset, params_sampling=sampling_params, degrees=degrees,
        binning=binning, form=form, idx_bin=idx_bin,
        catalogue_type='sim', statistic_type='bispec')
    if binning is None:
        binning = Binning.from_parameter_set(paramset)
    if None in paramset['boxsize'].values():
        raise ValueError("A batch needs an explicit box size.")
    if None in paramset['ngrid'].values():
        pd = _as_dict(paramset)
        _set_ngrid_from_cutoff(pd)
        paramset['ngrid'] = pd['ngrid']
    norms, offsets = [], [0]
    ctx = _engine.context_for(device, *catalogues)
    params_c = _engine.make_params(paramset, '3pt')
    for cat in catalogues:
        cat.periodise(_boxsize(paramset))
        if not _has_nz(cat):
            cat.compute_mean_density(boxsize=_boxsize(paramset))
        offsets.append(offsets[-1] + cat.ntotal)
        if paramset['norm_convention'] == 'mesh':
            norms.append(_norm_mesh(ctx, params_c,
                                    _engine.catalogue_arg(cat).c, 1., 3))
        else:
            norms.append(_norm_factor(paramset, ctx, params_c, None, cat, 1.,
                                      3))
    if any(isinstance(c, DeviceCatalogue) for c in catalogues):
        allc = _engine.catalogue_arg(DeviceCatalogue.concatenate(
            catalogues, device=ctx.device))
    else:
        cols = [np.concatenate(c) for c in
                zip(*(cat._columns() for cat in catalogues))]
        allc = _engine.HostCatalogue(*cols)
    return _engine.call_bispec_batch(
        ctx, params_c, allc.c, offsets, binning, norms,
        shape=paramset['shape'], idx_bin=paramset.get('idx_bin') or 0)


def compute_3pcf_in_gpp_box(catalogue_data, degrees=None, binning=None,
                            form=None, idx_bin=None, sampling_params=None,
                            paramset=None, save=False, logger=None,
                            device=None):
    """3PCF from a periodic-box catalogue (threept.py:1726-1830)."""
    return _compute_3pt_stats_sim_like(
        '3pcf', catalogue_data, paramset=paramset,
        params_sampling=sampling_params, degrees=degrees, binning=binning,
        form=form, idx_bin=idx_bin, save=save, logger=logger, device=device)
