"""Material pre-pass (csrc/material.cu, host code: runs without a GPU).

The padded grids equal a statement-by-statement NumPy restatement of
legacy/cpmlfdtd_cbindings.f95 bit for bit, for random images and tables
(real and complex permittivity, stiffness with and without the density
gradient, attenuation), and a hand-checked small case pins the carry rules:
the last interior row and column are overwritten by their neighbours, sig12
is not carried to high x, and low-z sig12 / sig23 take sig11 / sig33.
"""
import numpy as np
import pytest

from oracle import material_np as ref
from seidart_gpu import _lib
from seidart_gpu.fortran_io import read_record

pytestmark = pytest.mark.skipif(not _lib.LIB_PATH.exists(), reason="library not built")


def _case(seed, nx=13, nz=9, nmat=4, ncol=23, complex_valued=False):
    rng = np.random.default_rng(seed)
    im = rng.integers(1, nmat + 1, size=(nx, nz)).astype(np.int32)
    table = rng.uniform(1.0, 10.0, size=(nmat, ncol))
    if complex_valued:
        table = table + 1j * rng.uniform(-1.0, 1.0, size=(nmat, ncol))
    return im, table


@pytest.mark.parametrize("P", [0, 1, 3, 5])
def test_stiffness_matches_restatement(P):
    from seidart_gpu import material
    im, table = _case(P)
    grad = np.random.default_rng(9).uniform(0.5, 1.5, size=im.shape)
    for g in (None, grad):
        got = material.stiffness_arrays(im, table, P, g)
        want = ref.stiffness(im, table, P, g)
        for q, name in enumerate(material.STIFFNESS_NAMES):
            assert np.array_equal(got[name], want[q]), (name, P)


@pytest.mark.parametrize("P", [1, 2, 4])
@pytest.mark.parametrize("complex_valued", [False, True])
def test_permittivity_matches_restatement(P, complex_valued):
    from seidart_gpu import material
    im, table = _case(10 + P, ncol=13, complex_valued=complex_valued)
    got = material.permittivity_arrays(im, table, P, complex_valued)
    want = ref.permittivity(im, table, P, complex_valued)
    for q, name in enumerate(material.EPS_NAMES + material.SIG_NAMES):
        assert np.array_equal(got[name], want[q]), (name, P)


def test_attenuation_matches_restatement():
    from seidart_gpu import material
    im, table = _case(3, ncol=3)
    got = material.attenuation_arrays(im, table, 4, 12.5)
    want = ref.attenuation(im, table, 4, 12.5)
    for q, name in enumerate(material.GAMMA_NAMES):
        assert np.array_equal(got[name], want[q])


def test_carry_rules_on_a_small_case():
    from seidart_gpu import material
    nx, nz, P = 4, 3, 2
    im = np.array([[1, 2, 1], [2, 1, 2], [1, 1, 2], [2, 2, 1]], dtype=np.int32)  # (nx, nz)
    table = np.zeros((2, 13))
    table[:, 1:7] = [[1, 2, 3, 4, 5, 6], [10, 20, 30, 40, 50, 60]]        # eps
    table[:, 7:13] = [[.1, .2, .3, .4, .5, .6], [1., 2., 3., 4., 5., 6.]]  # sig
    g = material.permittivity_arrays(im, table, P)
    e11, s11, s12, s23, s33 = g["eps11"], g["sig11"], g["sig12"], g["sig23"], g["sig33"]
    # interior (0-based rows P..P+nx-1) except the last row, carried from its neighbour
    assert e11[P, P] == 1.0 and e11[P + 1, P] == 10.0
    assert np.array_equal(e11[nx + P - 1, :], e11[nx + P - 2, :])          # last interior row overwritten
    assert np.array_equal(e11[:, nz + P - 1], e11[:, nz + P - 2])          # last interior column overwritten
    assert np.array_equal(e11[0, :], e11[P, :])                            # low x carried
    # sig12 is not carried to high x: its high-x rows stay zero away from the z carry
    assert np.all(s12[nx + P:, P + 1:nz + P - 1] == 0.0)
    # low z: sig12 and sig23 take sig11's and sig33's column P+1 (1-based) -- the
    # last low-z statement (i = P+1) even replaces that first interior column
    assert np.array_equal(s12[:, P], s11[:, P]) and np.array_equal(s23[:, P], s33[:, P])
    # ... and column 1 is written in the first sweep, before sig11's high-x rows
    # beyond the last interior row are filled: those stay zero
    assert np.array_equal(s12[:nx + P, 0], s11[:nx + P, P]) and np.all(s12[nx + P:, 0] == 0.0)
    assert not np.array_equal(s12[P:nx + P - 1, P], table[im[:-1, 0] - 1, 8])  # not sig12's own values


def test_write_files_match_arrays(tmp_path):
    from seidart_gpu import material
    im, table = _case(5)
    material.stiffness_write(tmp_path, im, table, 3)
    arr = material.stiffness_arrays(im, table, 3)
    shape = arr["c11"].shape
    for name in ("c11", "c46", "rho"):
        rec = read_record(tmp_path / f"{name}.dat", np.float64).reshape(shape, order="F")
        assert np.array_equal(rec, arr[name])
    imc, tc = _case(6, ncol=13, complex_valued=True)
    material.permittivity_write(tmp_path, imc, tc, 2, complex_valued=True)
    arrc = material.permittivity_arrays(imc, tc, 2, complex_valued=True)
    rec = read_record(tmp_path / "eps13.dat", np.complex128).reshape(arrc["eps13"].shape, order="F")
    assert np.array_equal(rec, arrc["eps13"])
    rec = read_record(tmp_path / "sig22.dat", np.float64).reshape(arrc["sig22"].shape, order="F")
    assert np.array_equal(rec, arrc["sig22"])


def test_bad_material_id_is_rejected():
    from seidart_gpu import material
    from seidart_gpu._lib import SeidartError
    im, table = _case(7)
    im[2, 2] = 99
    with pytest.raises(SeidartError, match="not a table row"):
        material.stiffness_arrays(im, table, 2)


def test_legacy_module_writers(tmp_path, monkeypatch):
    """seidart_gpu.cpmlfdtd's writers take the binding's (im, mlist,
    npoints_pml, nx, nz) and read im from memory x fastest, like Fortran."""
    from seidart_gpu import cpmlfdtd, material
    im, table = _case(8)
    nx, nz = im.shape
    monkeypatch.chdir(tmp_path)
    cpmlfdtd.stiffness_write(np.asfortranarray(im).reshape(-1, order="F"), table, 2, nx, nz)
    want = material.stiffness_arrays(im, table, 2)
    rec = read_record(tmp_path / "c33.dat", np.float64).reshape(want["c33"].shape, order="F")
    assert np.array_equal(rec, want["c33"])
    cpmlfdtd.attenuation_write(np.asfortranarray(im).reshape(-1, order="F"), table[:, :3], 3, nx, nz, cpmlvalue=7.5)
    g = read_record(tmp_path / "gamma_x.dat", np.float64).reshape((nx + 6, nz + 6), order="F")
    assert g[0, 0] == 7.5
