"""The HDF5 dump reader and writer: the reference's golden dumps read back
as the committed fixtures, and files written here read back unchanged."""
import os

import numpy as np
import pytest

from puffin_gb300 import h5dump as H

GOLD = os.path.join(os.path.dirname(__file__), "golden", "f1main_expected.npz")
# the reference project's checkout, when there is one (its test/expected dumps)
REF = os.path.join(os.environ.get("PUFFIN_REFERENCE", ""), "test", "expected")


@pytest.mark.skipif(not os.environ.get("PUFFIN_REFERENCE") or not os.path.isdir(REF),
                    reason="set PUFFIN_REFERENCE to the reference checkout to read its dumps")
def test_reads_reference_dumps():
    g = np.load(GOLD)
    beam, attrs = H.read_particles(os.path.join(REF, "f1main_expected_electrons.h5"))
    for j, k in enumerate(H.PARTICLE_COLUMNS):
        np.testing.assert_array_equal(beam[k], g["electrons"][:, j])
    assert int(attrs["iCsteps"]) == 30
    re, im, shape, _ = H.read_field(os.path.join(REF, "f1main_expected_field.h5"))
    assert shape == (2, 511)
    np.testing.assert_array_equal(re, g["aperp"][0])
    np.testing.assert_array_equal(im, g["aperp"][1])


def test_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    beam = {k: rng.standard_normal(1000) for k in H.PARTICLE_COLUMNS}
    attrs = {"iCsteps": 1234, "zbarTotal": 0.75, "istep": 17, "zbarLocal": 0.125}
    H.write_particles(tmp_path / "e.h5", beam, attrs)
    b2, a2 = H.read_particles(tmp_path / "e.h5")
    for k in beam:
        np.testing.assert_array_equal(b2[k], beam[k])
    assert {k: a2[k] for k in attrs} == attrs
    mesh = (5, 4, 9)
    re, im = rng.standard_normal(180), rng.standard_normal(180)
    H.write_field(tmp_path / "f.h5", re, im, mesh, {"zbarTotal": 0.75})
    r2, i2, shape, fa = H.read_field(tmp_path / "f.h5")
    assert shape == (2, 9, 4, 5) and fa["zbarTotal"] == 0.75
    np.testing.assert_array_equal(r2, re)
    np.testing.assert_array_equal(i2, im)
    # several datasets in one file
    H.write(tmp_path / "m.h5", {"a": (np.arange(6.0).reshape(2, 3), {"k": 1}),
                                "b": (np.ones(4), {})})
    r = H.H5Reader(tmp_path / "m.h5")
    m = r.group_members(r.root_hdr)
    assert sorted(m) == ["a", "b"]
    np.testing.assert_array_equal(r.dataset(m["a"]), np.arange(6.0).reshape(2, 3))
