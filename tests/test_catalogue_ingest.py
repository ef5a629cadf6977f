"""CPU checks of the catalogue-ingestion oracle and of the host-side
plumbing around device catalogues (no GPU needed).

The oracle's text loader (a restatement of ``load_catalogue_file``,
particles.cpp:94-510) is pinned against ``np.loadtxt`` on the reference's
own test catalogue and on synthetic files with comments, blank lines,
permuted and extra columns and "::"-joined sub-files."""
import numpy as np
import pytest

from conftest import GOLDEN
from oracle import trv_oracle as O
from triumvirate_gb300 import _engine
from triumvirate_gb300.catalogue import ParticleCatalogue


def write_catalogue(path, cols, header=True, fmt=repr):
    lines = ["# x y z nz"] if header else []
    for row in zip(*cols):
        lines.append("  ".join(fmt(float(v)) for v in row))
        if len(lines) % 7 == 0:
            lines.append("")
            lines.append("# interleaved comment")
    path.write_text("\n".join(lines) + "\n")


def test_oracle_loader_matches_loadtxt_on_reference_catalogue():
    path = GOLDEN / "test_data_catalogue.txt"
    ref = np.loadtxt(path)
    got = O.load_catalogue_text(str(path), "x,y,z,nz")
    for i, f in enumerate(['x', 'y', 'z', 'nz']):
        assert np.array_equal(got[f], ref[:, i]), f
    assert np.array_equal(got['ws'], np.ones(3))
    assert np.array_equal(got['w'], np.ones(3))


def test_oracle_loader_subfiles_permuted_columns_and_defaults(tmp_path):
    rng = np.random.default_rng(7)
    a = rng.uniform(-500., 500., size=(5, 40))
    b = rng.uniform(-500., 500., size=(5, 25))
    pa, pb = tmp_path / "a.txt", tmp_path / "b.txt"
    write_catalogue(pa, a)
    write_catalogue(pb, b, fmt=lambda v: f"{v:.6e}")
    # Columns: id, z, x, ws, y (no nz, no wc).
    got = O.load_catalogue_text(f"{pa}::{pb}", "id,z,x,ws,y", volume=1.e9)
    both = np.concatenate([np.loadtxt(pa), np.loadtxt(pb)])
    assert np.array_equal(got['z'], both[:, 1])
    assert np.array_equal(got['x'], both[:, 2])
    assert np.array_equal(got['ws'], both[:, 3])
    assert np.array_equal(got['y'], both[:, 4])
    assert np.array_equal(got['wc'], np.ones(65))
    assert np.array_equal(got['nz'], np.full(65, 65 / 1.e9))
    assert np.array_equal(got['w'], both[:, 3])


def test_oracle_box_preparation_restatements():
    rng = np.random.default_rng(3)
    x, y, z = rng.uniform(-600., 700., size=(3, 1000))
    box = [1000., 1100., 1200.]
    # offset_coords_for_periodicity leaves [0, L) alone and folds the rest.
    wx, wy, wz = O.offset_coords_for_periodicity(x, y, z, box)
    for w, c, L in zip((wx, wy, wz), (x, y, z), box):
        inside = (c >= 0.) & (c < L)
        assert np.array_equal(w[inside], c[inside])
        assert np.all((w >= 0.) & (w <= L))
    # Python and C++ padding agree up to the association of one product.
    p, o = O.pad(x, y, z, box, ngrid=[64] * 3, ngrid_pad=[2.] * 3)
    q, oc = O.pad_cpp(x, y, z, box, ngrid=[64] * 3, ngrid_pad=[2.] * 3)
    assert np.allclose(o, oc, rtol=1e-15, atol=1e-12)
    assert np.allclose(p[0], q[0], rtol=0, atol=1e-12)


def test_host_catalogue_argument_keeps_lines_of_sight():
    rng = np.random.default_rng(1)
    d = rng.uniform(1., 2., size=(4, 10))
    cat = ParticleCatalogue(d[0], d[1], d[2], nz=d[3])
    arg = _engine.catalogue_arg(cat, with_los=True)
    assert arg.c.n == 10 and arg.c.los_x
    assert np.allclose(arg.los[0], cat.compute_los()[:, 0])
    bare = _engine.catalogue_arg(cat)
    assert not bare.c.los_x
