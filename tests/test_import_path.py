"""The reference's import path: ``triumvirate.*`` forwards to this
package, and the estimators report their stages to a given logger."""
import logging

import numpy as np
import pytest

import triumvirate_gb300.catalogue as gc
import triumvirate_gb300.dataobjs as gd
import triumvirate_gb300.parameters as gp
import triumvirate_gb300.threept as gt
import triumvirate_gb300.transforms as gf
import triumvirate_gb300.twopt as gw


def test_reference_import_path_forwards():
    from triumvirate import (catalogue, dataobjs, parameters, threept,
                             transforms, twopt)
    for mod, src, names in [
            (threept, gt, ['compute_bispec', 'compute_bispec_in_gpp_box',
                           'compute_3pcf', 'compute_3pcf_in_gpp_box',
                           'compute_3pcf_window']),
            (twopt, gw, ['compute_powspec', 'compute_powspec_in_gpp_box']),
            (catalogue, gc, ['ParticleCatalogue']),
            (parameters, gp, ['ParameterSet', 'fetch_paramset_template']),
            (dataobjs, gd, ['Binning']),
            (transforms, gf, ['SphericalBesselTransform',
                              'DoubleSphericalBesselTransform',
                              'resample_lglin', 'resample_lin'])]:
        for name in names:
            assert getattr(mod, name) is getattr(src, name), name


def test_setup_logger_has_stat_level(capsys):
    from triumvirate.logger import setup_logger
    lg = setup_logger()
    lg.stat("stage %d", 1)
    lg.debug("hidden")
    out = capsys.readouterr().out
    assert "STAT GB300] stage 1" in out and "hidden" not in out


@pytest.mark.gpu
def test_estimator_logs_its_stages(caplog):
    from triumvirate.catalogue import ParticleCatalogue
    from triumvirate.dataobjs import Binning
    from triumvirate.threept import compute_bispec_in_gpp_box
    rng = np.random.default_rng(3)
    x, y, z = rng.uniform(0., 500., size=(3, 2000))
    logger = logging.getLogger('trv-test')
    with caplog.at_level(logging.INFO, logger='trv-test'):
        compute_bispec_in_gpp_box(
            ParticleCatalogue(x, y, z, nz=2000 / 500. ** 3),
            degrees=(0, 0, 0), binning=Binning('fourier', 'lin', 0.02, 0.1,
                                               3),
            form='diag', sampling_params={'boxsize': [500.] * 3,
                                          'ngrid': [32] * 3},
            logger=logger)
    text = caplog.text
    for msg in ("Parameter set have been initialised.",
                "Catalogue box has been periodised.",
                "Normalisation factor:", "Measuring bispectrum",
                "... measured bispectrum"):
        assert msg in text, msg
