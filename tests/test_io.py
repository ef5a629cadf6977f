"""Measurement files: the reader against the library's own golden files, and
the writer reproducing their rows and header lines byte for byte."""
import numpy as np
import pytest

from conftest import GOLDEN
from triumvirate_gb300 import io
from triumvirate_gb300.catalogue import ParticleCatalogue
from triumvirate_gb300.parameters import ParameterSet, fetch_paramset_template

CASES = {
    'bk000_diag_gpp.txt': ('bispec', (0, 0, 0), 'diag', None),
    'bk202_diag_lpp.txt': ('bispec', (2, 0, 2), 'diag', None),
    'bk000_row0_gpp.txt': ('bispec', (0, 0, 0), 'row', 0),
    'zeta000_diag_gpp.txt': ('3pcf', (0, 0, 0), 'diag', None),
    'zeta202_diag_lpp.txt': ('3pcf', (2, 0, 2), 'diag', None),
    'pk0_gpp.txt': ('powspec', (0, 0, 0), 'full', None),
    'pk2_lpp.txt': ('powspec', (0, 0, 2), 'full', None),
}


def _paramset(stat, degrees, form, idx_bin, tag, odir=None):
    d = fetch_paramset_template('dict')
    d['boxsize'] = {ax: 1000. for ax in 'xyz'}
    d['ngrid'] = {ax: 64 for ax in 'xyz'}
    d['statistic_type'] = stat
    d['degrees'] = dict(zip(['ell1', 'ell2', 'ELL'], degrees))
    d['form'] = form
    d['idx_bin'] = idx_bin
    d['tags']['output'] = tag
    d['directories']['measurements'] = odir
    d['range'] = [0.005, 0.105]
    d['num_bins'] = 4
    return ParameterSet(param_dict=d)


def _norms(header):
    line = next(h for h in header
                if h.startswith('Normalisation factor alternatives'))
    vals = [float(t.split(' (')[0]) for t in line.split(': ')[1].split(', ')]
    return vals


@pytest.mark.parametrize("name", sorted(CASES))
def test_reader_matches_loadtxt(name):
    out = io.read_measurements(GOLDEN / name)
    tab = np.loadtxt(GOLDEN / name)
    stat = CASES[name][0]
    if stat == 'powspec':
        assert np.array_equal(out['kbin'], tab[:, 0])
        assert np.array_equal(out['nmodes'], tab[:, 2].astype(np.int64))
        assert np.array_equal(out['pk_raw'], tab[:, 3] + 1j * tab[:, 4])
        assert np.array_equal(out['pk_shot'], tab[:, 5] + 1j * tab[:, 6])
    else:
        v = 'bk' if stat == 'bispec' else 'zeta'
        c = 'k' if stat == 'bispec' else 'r'
        n = 'nmodes' if stat == 'bispec' else 'npairs'
        assert np.array_equal(out[f'{c}1_eff'], tab[:, 1])
        assert np.array_equal(out[f'{n}_2'], tab[:, 5].astype(np.int64))
        assert np.array_equal(out[f'{v}_raw'], tab[:, 6] + 1j * tab[:, 7])
        assert np.array_equal(out[f'{v}_shot'], tab[:, 8] + 1j * tab[:, 9])
    assert out['header'][-7].startswith('Box size')


@pytest.mark.parametrize("name", sorted(CASES))
def test_writer_reproduces_golden_layout(name, tmp_path):
    stat, degrees, form, idx_bin = CASES[name]
    golden = (GOLDEN / name).read_text().splitlines()
    res = io.read_measurements(GOLDEN / name)
    header = res.pop('header')
    tag = '_' + name.rsplit('_', 1)[1][:-4]
    ps = _paramset(stat, degrees, form, idx_bin, tag, str(tmp_path))
    assert io.measurement_filename(ps) == name[:-4]
    part, mesh, mixed = _norms(header)
    # Catalogue lines from the golden, the rest from this writer.
    text = "\n".join(header[:-7] +
                     [io.measurement_header(ps, part, mesh, mixed)])
    path = io.save_measurements(res, ps, '.txt', text)
    assert path.name == name
    assert path.read_text().splitlines() == golden


def test_npz_round_trip(tmp_path):
    res = io.read_measurements(GOLDEN / 'bk000_diag_gpp.txt')
    res.pop('header')
    ps = _paramset('bispec', (0, 0, 0), 'diag', None, '_x', str(tmp_path))
    path = io.save_measurements(res, ps, '.npz', 'a\nb')
    back = io.read_measurements(path)
    assert back['header'] == ['a', 'b']
    for k, v in res.items():
        assert np.array_equal(back[k], v)


def test_catalogue_header_lines():
    pos = np.loadtxt(GOLDEN / 'test_data_catalogue.txt')
    cat = ParticleCatalogue(pos[:, 0], pos[:, 1], pos[:, 2], nz=pos[:, 3])
    # The library writes the header after periodising into the box.
    cat.periodise([1000.] * 3)
    golden = [ln[2:] for ln in
              (GOLDEN / 'bk000_diag_gpp.txt').read_text().splitlines()[1:3]]
    assert cat.write_attrs_as_header().splitlines()[1:] == golden
    two = cat.write_attrs_as_header(catalogue_ref=cat).splitlines()
    assert [ln.split(':')[0] for ln in two] == [
        'Data catalogue source', 'Data catalogue size',
        'Data-source particle extents', 'Random catalogue source',
        'Random catalogue size', 'Random-source particle extents']


def test_unknown_format_raises(tmp_path):
    ps = _paramset('bispec', (0, 0, 0), 'diag', None, '', str(tmp_path))
    with pytest.raises(ValueError, match="Unrecognised save format"):
        io.save_measurements({}, ps, '.csv', '')
