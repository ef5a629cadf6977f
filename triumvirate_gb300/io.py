"""Measurement files in the library's layouts: the tab-separated text table
with a '#' header, and the .npz archive (threept.py:196-364 and 707-735,
twopt.py:158-318 and 633-663; the C++ writers io.cpp:102-300 and 444-555
produce the same columns).

Text tables
    header = catalogue attributes (catalogue.py:803-858), then box, mesh,
    assignment and normalisation lines, then the column index line
    "[0] k1_cen, [1] k1_eff, ...";
    rows = centre, effective coordinate (%.9e) and count (%10d) per bin
    coordinate, then real and imaginary parts (% .9e) of the raw and
    shot-noise values.
.npz
    the results dictionary plus its 'header' string.

``read_measurements`` inverts both: it returns the results dictionary
under the keys the estimators return, complex values reassembled, and the
header lines under 'header'.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

# Result keys per (points, space): coordinate blocks then value keys.
_KEYS = {
    ('3pt', 'fourier'): (['k1_bin', 'k1_eff', 'nmodes_1',
                          'k2_bin', 'k2_eff', 'nmodes_2'],
                         ['bk_raw', 'bk_shot']),
    ('3pt', 'config'): (['r1_bin', 'r1_eff', 'npairs_1',
                         'r2_bin', 'r2_eff', 'npairs_2'],
                        ['zeta_raw', 'zeta_shot']),
    ('2pt', 'fourier'): (['kbin', 'keff', 'nmodes'], ['pk_raw', 'pk_shot']),
    ('2pt', 'config'): (['rbin', 'reff', 'npairs'], ['xi']),
}

# Column names of the text header for the same layouts.
_COLS = {
    ('3pt', 'fourier'): ['k1_cen', 'k1_eff', 'nmodes_1',
                         'k2_cen', 'k2_eff', 'nmodes_2'],
    ('3pt', 'config'): ['r1_cen', 'r1_eff', 'npairs_1',
                        'r2_cen', 'r2_eff', 'npairs_2'],
    ('2pt', 'fourier'): ['k_cen', 'k_eff', 'nmodes'],
    ('2pt', 'config'): ['r_cen', 'r_eff', 'npairs'],
}


def _layout(paramset):
    npoint, space = paramset['npoint'], paramset['space']
    if (npoint, space) not in _KEYS:
        raise ValueError(
            "`paramset` 'statistic_type' does not correspond to a "
            "recognised clustering statistic.")
    return npoint, space


def _multipole(paramset):
    deg = paramset['degrees']
    if paramset['npoint'] == '3pt':
        return "{ell1}{ell2}{ELL}".format(**deg)
    return "{:d}".format(deg['ELL'])


def measurement_filename(paramset):
    """File name without suffix (threept.py:196-242, twopt.py:158-192)."""
    npoint, _ = _layout(paramset)
    tag = paramset['tags'].get('output') or ""
    multipole = _multipole(paramset)
    stat = paramset['statistic_type']
    if npoint == '2pt':
        prefix = {'powspec': 'pk', '2pcf': 'xi', '2pcf-win': 'xiw'}.get(stat)
        if prefix is None:
            raise ValueError(
                "`paramset` 'statistic_type' does not correspond to a "
                "recognised two-point statistic.")
        return f"{prefix}{multipole}{tag}"
    form = paramset['form']
    binform = {'diag': "_diag", 'full': "_full"}.get(form)
    if form == 'off-diag':
        binform = "_offdiag{:d}".format(paramset['idx_bin'])
    elif form == 'row':
        binform = "_row{:d}".format(paramset['idx_bin'])
    prefix = {'bispec': 'bk', '3pcf': 'zeta', '3pcf-win': 'zetaw'}.get(stat)
    if prefix is None:
        raise ValueError(
            "`paramset` 'statistic_type' does not correspond to a "
            "recognised three-point statistic.")
    return f"{prefix}{multipole}{binform}{tag}"


def _value_columns(paramset):
    npoint, space = _layout(paramset)
    m = _multipole(paramset)
    if npoint == '3pt':
        v = 'bk' if space == 'fourier' else 'zeta'
        return [f"Re{{{v}{m}_raw}}", f"Im{{{v}{m}_raw}}",
                f"Re{{{v}{m}_shot}}", f"Im{{{v}{m}_shot}}"]
    if space == 'fourier':
        return [f"Re{{pk{m}_raw}}", f"Im{{pk{m}_raw}}",
                f"Re{{pk{m}_shot}}", f"Im{{pk{m}_shot}}"]
    return [f"Re{{xi{m}}}", f"Im{{xi{m}}}"]


def measurement_header(paramset, norm_factor_part, norm_factor_mesh,
                       norm_factor_meshes=0.):
    """Sampling, normalisation and column lines (threept.py:245-328,
    twopt.py:195-274)."""
    npoint, space = _layout(paramset)
    conv = paramset['norm_convention']
    norm = {'none': 1., 'particle': norm_factor_part,
            'mesh': norm_factor_mesh,
            'mesh-mixed': norm_factor_meshes}[conv]
    cols = _COLS[(npoint, space)] + _value_columns(paramset)
    mixed = "mesh-mixed; n/a" if npoint == '3pt' else "mesh-mixed"
    box = [paramset['boxsize'][ax] for ax in 'xyz']
    ngrid = [paramset['ngrid'][ax] for ax in 'xyz']
    lines = [
        "Box size: [{:.3f}, {:.3f}, {:.3f}]".format(*box),
        "Box alignment: {}".format(paramset['alignment']),
        "Mesh number: [{:d}, {:d}, {:d}]".format(*ngrid),
        "Mesh assignment and interlacing: {}, {}".format(
            paramset['assignment'], paramset['interlace']),
        "Normalisation factor: {:.9e} ({})".format(norm, conv),
        "Normalisation factor alternatives: "
        "{:.9e} (particle), {:.9e} (mesh), {:.9e} ({})".format(
            norm_factor_part, norm_factor_mesh, norm_factor_meshes, mixed),
        ", ".join("[{:d}] {}".format(i, c) for i, c in enumerate(cols)),
    ]
    return "\n".join(lines)


def measurement_datatab(results, paramset):
    """Rows of the text table (threept.py:331-364, twopt.py:277-318)."""
    coord_keys, value_keys = _KEYS[_layout(paramset)]
    cols = [results[k] for k in coord_keys]
    for k in value_keys:
        v = np.asarray(results[k])
        cols += [v.real, v.imag]
    return np.transpose(cols)


def _datafmt(paramset):
    npoint, _ = _layout(paramset)
    ncoord = 2 if npoint == '3pt' else 1
    nval = len(_value_columns(paramset))
    return '\t'.join((['%.9e'] * 2 + ['%10d']) * ncoord + ['% .9e'] * nval)


def save_measurements(results, paramset, save, header):
    """Write `results` as '.txt' or '.npz' into the measurement directory
    under `measurement_filename`; returns the path written."""
    odir = paramset['directories'].get('measurements') or ""
    path = Path(odir, measurement_filename(paramset))
    if str(save).lower() == '.txt':
        path = path.with_suffix('.txt')
        np.savetxt(path, measurement_datatab(results, paramset),
                   fmt=_datafmt(paramset), header=header, delimiter='\t')
    elif str(save).lower().endswith('.npz'):
        path = path.with_suffix('.npz')
        np.savez(path, header=header, **results)
    else:
        raise ValueError(
            f"Unrecognised save format for measurements: {save}.")
    return path


def read_measurements(path):
    """Results dictionary of a measurement file written by the library."""
    path = Path(path)
    if path.suffix == '.npz':
        with np.load(path) as f:
            out = {k: f[k] for k in f.files}
        out['header'] = str(out['header']).splitlines()
        return out
    header = []
    with open(path) as f:
        for line in f:
            if not line.startswith('#'):
                break
            header.append(line[1:].strip())
    colnames = [c.split('] ', 1)[1] for c in header[-1].split(', ')]
    tab = np.loadtxt(path, ndmin=2)
    if tab.shape[1] != len(colnames):
        raise ValueError(f"{path}: {tab.shape[1]} columns, header names "
                         f"{len(colnames)}.")
    first = colnames[0]
    layout = {'k1_cen': ('3pt', 'fourier'), 'r1_cen': ('3pt', 'config'),
              'k_cen': ('2pt', 'fourier'), 'r_cen': ('2pt', 'config')}
    if first not in layout:
        raise ValueError(f"{path}: unrecognised column '{first}'.")
    coord_keys, value_keys = _KEYS[layout[first]]
    out = {}
    for i, k in enumerate(coord_keys):
        col = tab[:, i]
        out[k] = col.astype(np.int64) if k.startswith(('nmodes', 'npairs')) \
            else col
    j = len(coord_keys)
    for k in value_keys:
        out[k] = tab[:, j] + 1j * tab[:, j + 1]
        j += 2
    out['header'] = header
    return out
