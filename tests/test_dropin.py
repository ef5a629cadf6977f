"""The C++ drop-in layer (include/trv_dropin.hpp, libtrv_dropin.so): a
program written against the reference's trv:: interface, built by
triumvirate_gb300/build.py, reproduces the reference's golden file.

Without a GPU: the library exports the reference's C++ entry points and
parameter errors raise the reference's exception types.  On the GPU: the
program's B_000 diag of the reference tests' 3-particle catalogue matches
``bk000_diag_gpp.txt`` within the reference test's tolerance, and the
Python entry point on the same inputs to 1e-12."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import BOX, GOLDEN, KBINS, NMESH, load_golden
from triumvirate_gb300 import build as B

ENTRY_POINTS = [
    'compute_bispec_in_gpp_box', 'compute_bispec', 'compute_3pcf',
    'compute_3pcf_in_gpp_box', 'compute_3pcf_window', 'compute_powspec',
    'compute_powspec_in_gpp_box', 'calc_bispec_normalisation_from_particles',
    'calc_bispec_normalisation_from_mesh',
    'calc_powspec_normalisation_from_particles',
    'calc_powspec_normalisation_from_mesh',
    'ParticleCatalogue::load_catalogue_file',
    'ParticleCatalogue::offset_coords_for_periodicity',
    'ParticleCatalogue::centre_in_box', 'ParameterSet::validate',
    'Binning::set_bins']


@pytest.fixture(scope='module')
def program():
    B.build()
    assert B.DROPIN_LIB.exists() and B.DROPIN_TEST.exists()
    return B.DROPIN_TEST


def test_dropin_library_exports_reference_entry_points(program):
    r = subprocess.run(['nm', '-DC', '--defined-only', str(B.DROPIN_LIB)],
                       capture_output=True, text=True, check=True)
    for name in ENTRY_POINTS:
        assert f"trv::{name}(" in r.stdout, name


def test_dropin_errors_map_to_reference_exceptions(program):
    r = subprocess.run([str(program), '--errors'], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert 'InvalidParameterError' in r.stdout
    assert 'InvalidDataError' in r.stdout


def _run(program, precision):
    r = subprocess.run([str(program), str(GOLDEN / 'test_data_catalogue.txt'),
                        precision], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    return np.loadtxt(r.stdout.splitlines(), ndmin=2).T


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ['fp64', 'fp32mixed'])
def test_dropin_program_matches_golden(program, precision):
    got = _run(program, precision)
    ext = load_golden('bk000_diag_gpp.txt')
    for i in range(6):
        assert np.allclose(got[i], ext[i]), i
    raw, shot = got[6] + 1j * got[7], got[8] + 1j * got[9]
    assert np.allclose(raw, ext[6] + 1j * ext[7])
    assert np.allclose(shot, ext[8] + 1j * ext[9], atol=1e-6)


@pytest.mark.gpu
def test_dropin_program_matches_python_entry_point(program,
                                                   data_catalogue_array):
    from triumvirate_gb300.catalogue import ParticleCatalogue
    from triumvirate_gb300.dataobjs import Binning
    from triumvirate_gb300.threept import compute_bispec_in_gpp_box
    d = data_catalogue_array
    res = compute_bispec_in_gpp_box(
        ParticleCatalogue(d[:, 0], d[:, 1], d[:, 2], nz=d[:, 3]),
        degrees=(0, 0, 0), binning=Binning('fourier', 'lin', *KBINS),
        form='diag',
        sampling_params={'boxsize': [BOX] * 3, 'ngrid': [NMESH] * 3,
                         'assignment': 'tsc', 'precision': 'fp64'})
    got = _run(program, 'fp64')
    assert np.array_equal(got[2].astype(int), res['nmodes_1'])
    for k, (a, b) in (('bk_raw', (6, 7)), ('bk_shot', (8, 9))):
        c = got[a] + 1j * got[b]
        assert np.all(np.abs(c - res[k]) <= 1e-12 * np.abs(res[k])), k
