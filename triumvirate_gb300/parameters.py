"""Parameter sets (mirrors ``triumvirate.parameters``, parameters.pyx, and
the derivations of ``trv::ParameterSet::validate``, parameters.cpp:466-1270).

The dictionary layout is the reference's YAML template
(``resources/params_template.yml``) plus one key, ``precision``
(``'fp64'`` or ``'fp32mixed'``), choosing the arithmetic of meshes and
transforms on the GPU.
"""
from __future__ import annotations

import copy
from pathlib import Path

import numpy as np

_TEMPLATE = {
    'directories': {'catalogues': None, 'measurements': None},
    'files': {'data_catalogue': None, 'rand_catalogue': None},
    'catalogue_columns': [],
    'catalogue_dataset': None,
    'tags': {'output': None},
    'boxsize': {'x': None, 'y': None, 'z': None},
    'ngrid': {'x': None, 'y': None, 'z': None},
    'expand': 1.,
    'cutoff_nyq': None,
    'alignment': 'centre',
    'padscale': 'box',
    'padfactor': None,
    'assignment': 'tsc',
    'interlace': False,
    'catalogue_type': None,
    'statistic_type': None,
    'degrees': {'ell1': None, 'ell2': None, 'ELL': None},
    'wa_orders': {'i': None, 'j': None},
    'form': 'diag',
    'norm_convention': 'particle',
    'binning': 'lin',
    'range': [None, None],
    'num_bins': None,
    'idx_bin': None,
    'fftw_scheme': 'measure',
    'use_fftw_wisdom': False,
    'save_binned_vectors': False,
    'verbose': 20,
    'progbar': False,
    'precision': 'fp64',
}

_ORDERS = {'ngp': 1, 'cic': 2, 'tsc': 3, 'pcs': 4}

# statistic_type -> (npoint, space)  (parameters.cpp:780-822)
_STAT_TYPES = {
    'powspec': ('2pt', 'fourier'),
    '2pcf': ('2pt', 'config'),
    '2pcf-win': ('2pt', 'config'),
    'bispec': ('3pt', 'fourier'),
    '3pcf': ('3pt', 'config'),
    '3pcf-win': ('3pt', 'config'),
    '3pcf-win-wa': ('3pt', 'config'),
    'modes': ('none', 'fourier'),
    'pairs': ('none', 'config'),
}


class InvalidParameterError(ValueError):
    """Invalid parameter (``trv::sys::InvalidParameterError``)."""


def fetch_paramset_template(format, ret_defaults=False):
    """Parameter-set template as a dict (parameters.pyx:612-667).

    ``format='text'`` returns a YAML rendering of the same template.
    """
    tmpl = copy.deepcopy(_TEMPLATE)
    defaults = {k: v for k, v in tmpl.items()
                if not isinstance(v, (tuple, list, set, dict))
                and v is not None}
    if format.lower() == 'dict':
        return (tmpl, defaults) if ret_defaults else tmpl
    if format.lower() == 'text':
        text = _to_yaml(tmpl)
        return (text, defaults) if ret_defaults else text
    raise ValueError("`format` must be either 'text' or 'dict'.")


def _to_yaml(d, indent=0):
    lines = ["---"] if indent == 0 else []
    for k, v in d.items():
        pad = "  " * indent
        if isinstance(v, dict):
            lines.append(f"{pad}{k}:")
            lines.append(_to_yaml(v, indent + 1))
        else:
            val = "" if v is None else ("[~, ~]" if v == [None, None]
                                        else str(v).lower()
                                        if isinstance(v, bool) else str(v))
            lines.append(f"{pad}{k}: {val}".rstrip())
    if indent == 0:
        lines.append("...")
    return "\n".join(lines)


class ParameterSet:
    """Parameter set (``triumvirate.parameters.ParameterSet``).

    Parameters
    ----------
    param_filepath : str or path-like, optional
        YAML parameter file (needs PyYAML).
    param_dict : dict, optional
        Parameter dictionary (template layout).
    logger : logging.Logger, optional
        Logger.
    """

    def __init__(self, param_filepath=None, param_dict=None, logger=None):
        if param_filepath is not None and param_dict is not None:
            raise ValueError("Cannot set both `param_filepath` and "
                             "`param_dict`.")
        if param_filepath is None and param_dict is None:
            raise ValueError("Either `param_filepath` or `param_dict` "
                             "must be set.")
        self._logger = logger
        if param_filepath is not None:
            try:
                import yaml
            except ImportError as e:  # pragma: no cover - env dependent
                raise ImportError("Reading a YAML parameter file needs "
                                  "PyYAML; pass `param_dict` instead.") from e
            with open(Path(param_filepath)) as f:
                param_dict = yaml.load(f, Loader=yaml.SafeLoader)
        self._params = copy.deepcopy(param_dict)
        for key, val in _TEMPLATE.items():
            self._params.setdefault(key, copy.deepcopy(val))
        self._validate()

    # dict-like access
    def __getitem__(self, key):
        return self._params[key]

    def __setitem__(self, key, val):
        self._params[key] = val
        self._validate()

    def get(self, key, default=None):
        return self._params.get(key, default)

    def items(self):
        return self._params.items()

    def keys(self):
        return self._params.keys()

    def update(self, *args, **kwargs):
        self._params.update(*args, **kwargs)
        self._validate()

    def __repr__(self):
        return f"ParameterSet({self._params!r})"

    def _validate(self, init=False):
        """Derived parameters (parameters.cpp:466-1270, on-path subset)."""
        p = self._params
        assignment = p.get('assignment')
        if assignment not in _ORDERS:
            raise InvalidParameterError(
                "Mesh assignment scheme must be 'ngp', 'cic', 'tsc' or "
                f"'pcs': `assignment` = '{assignment}'.")
        p['assignment_order'] = _ORDERS[assignment]
        interlace = p.get('interlace')
        if isinstance(interlace, str):
            interlace = interlace.lower() in ('true', 'on', 'yes')
        p['interlace'] = bool(interlace)
        st = p.get('statistic_type')
        if st is not None:
            if st not in _STAT_TYPES:
                raise InvalidParameterError(
                    f"Statistic type is not recognised: `statistic_type` = "
                    f"'{st}'.")
            p['npoint'], p['space'] = _STAT_TYPES[st]
        else:
            p.setdefault('npoint', None)
            p.setdefault('space', None)
        form = p.get('form')
        if form not in ('full', 'diag', 'off-diag', 'row'):
            raise InvalidParameterError(
                "Three-point statistic form is not recognised: `form` = "
                f"'{form}'.")
        ell1 = p['degrees'].get('ell1')
        ell2 = p['degrees'].get('ell2')
        p['shape'] = 'triu' if (form == 'full' and ell1 == ell2) else form
        if p.get('npoint') == '3pt' and p['interlace']:
            p['interlace'] = False   # parameters.cpp:1240-1249
        if p.get('norm_convention') not in ('none', 'particle', 'mesh',
                                            'mesh-mixed'):
            raise InvalidParameterError(
                "Normalisation convention must be 'none', 'particle', "
                "'mesh' or 'mesh-mixed'.")
        if p.get('precision') not in ('fp64', 'fp32mixed'):
            raise InvalidParameterError(
                "`precision` must be 'fp64' or 'fp32mixed'.")
        bs = p['boxsize']
        if None not in bs.values():
            p['volume'] = float(bs['x']) * float(bs['y']) * float(bs['z'])
        ng = p['ngrid']
        if None not in ng.values():
            p['nmesh'] = int(ng['x']) * int(ng['y']) * int(ng['z'])
        self._validity = True


def _modify_sampling_parameters(paramset, params_sampling=None,
                                params_default=None, ret_defaults=False):
    """Override sampling parameters (parameters.pyx:669-789)."""
    if params_sampling is None:
        return (paramset, params_default) if ret_defaults else paramset

    def drop(*keys):
        if params_default:
            for k in keys:
                params_default.pop(k, None)

    for key in ('expand', 'alignment', 'assignment', 'interlace',
                'cutoff_nyq'):
        if key in params_sampling:
            paramset[key] = params_sampling[key]
            drop(key)
    if paramset.get('alignment') == 'pad' and \
            'boxpad' in params_sampling and 'gridpad' in params_sampling:
        raise ValueError(
            "Cannot set both 'boxpad` and 'gridpad' in `params_sampling`.")
    if 'boxpad' in params_sampling:
        paramset['padscale'] = 'box'
        paramset['padfactor'] = params_sampling['boxpad']
        drop('padscale', 'padfactor')
    if 'gridpad' in params_sampling:
        paramset['padscale'] = 'grid'
        paramset['padfactor'] = params_sampling['gridpad']
        drop('padscale', 'padfactor')
    for key in ('boxsize', 'ngrid'):
        if key in params_sampling:
            val = params_sampling[key]
            if np.isscalar(val):
                val = [val] * 3
            paramset[key] = dict(zip(['x', 'y', 'z'], val))
            drop(key)
    if 'precision' in params_sampling:
        paramset['precision'] = params_sampling['precision']
    return (paramset, params_default) if ret_defaults else paramset


def _modify_measurement_parameters(paramset, params_measure=None,
                                   params_default=None, ret_defaults=False):
    """Override measurement parameters (parameters.pyx:792-863)."""
    if params_measure is None:
        return (paramset, params_default) if ret_defaults else paramset
    degrees = dict(paramset['degrees'])
    for k in ('ell1', 'ell2', 'ELL'):
        if k in params_measure:
            degrees[k] = params_measure[k]
    paramset['degrees'] = degrees
    wa = dict(paramset['wa_orders'])
    for k in ('i_wa', 'j_wa'):
        if k in params_measure:
            wa[k[0]] = params_measure[k]
    paramset['wa_orders'] = wa
    for k in ('idx_bin', 'form', 'num_bins'):
        if k in params_measure:
            paramset[k] = params_measure[k]
            if params_default:
                params_default.pop(k, None)
    rng = list(paramset['range'])
    if 'bin_min' in params_measure:
        rng[0] = params_measure['bin_min']
    if 'bin_max' in params_measure:
        rng[1] = params_measure['bin_max']
    paramset['range'] = rng
    return (paramset, params_default) if ret_defaults else paramset


def _set_ngrid_from_cutoff(paramset):
    """Mesh number from the Nyquist cutoff (parameters.pyx:866-900)."""
    ngrid = {}
    for ax in ['x', 'y', 'z']:
        if paramset['space'] == 'fourier':
            ngrid[ax] = int(np.ceil(
                paramset['boxsize'][ax] * paramset['cutoff_nyq'] / np.pi))
        elif paramset['space'] == 'config':
            ngrid[ax] = int(2 * np.ceil(
                paramset['boxsize'][ax] / paramset['cutoff_nyq']))
        else:
            raise ValueError("Space must be either 'fourier' or 'config': "
                             f"`space` = '{paramset['space']}'.")
        ngrid[ax] += ngrid[ax] % 2
    paramset['ngrid'] = ngrid
    return paramset


def _as_dict(paramset):
    if isinstance(paramset, ParameterSet):
        return copy.deepcopy(paramset._params)
    return copy.deepcopy(paramset)
