"""The material pre-pass on the device (seidart_*_arrays_dev): padded grids
equal to the statement-by-statement NumPy restatement of
legacy/cpmlfdtd_cbindings.f95:60-611 bit for bit (stiffness with and
without the density gradient, real and complex permittivity, attenuation),
and a seismic2 solver fed those device grids directly gives the same run as
one fed the host grids."""
import dataclasses

import numpy as np
import pytest

import seidart_gpu as sg
from oracle import material_np as ref
from seidart_gpu import material, models

pytestmark = pytest.mark.gpu


def _case(seed, nx=13, nz=9, nmat=4, ncol=23, complex_valued=False):
    rng = np.random.default_rng(seed)
    im = rng.integers(1, nmat + 1, size=(nx, nz)).astype(np.int32)
    table = rng.uniform(1.0, 10.0, size=(nmat, ncol))
    if complex_valued:
        table = table + 1j * rng.uniform(-1.0, 1.0, size=(nmat, ncol))
    return im, table


@pytest.mark.parametrize("P", [0, 1, 3, 5])
def test_device_stiffness_matches_restatement(P):
    im, table = _case(P)
    grad = np.random.default_rng(9).uniform(0.5, 1.5, size=im.shape)
    for g in (None, grad):
        got = material.stiffness_arrays_device(im, table, P, g)
        want = ref.stiffness(im, table, P, g)
        for q, name in enumerate(material.STIFFNESS_NAMES):
            assert np.array_equal(material.fortran(got[name]), want[q]), (name, P)


@pytest.mark.parametrize("P", [1, 2, 4])
@pytest.mark.parametrize("complex_valued", [False, True])
def test_device_permittivity_matches_restatement(P, complex_valued):
    im, table = _case(10 + P, nx=17, nz=11, ncol=13, complex_valued=complex_valued)
    got = material.permittivity_arrays_device(im, table, P, complex_valued)
    want = ref.permittivity(im, table, P, complex_valued)
    for q, name in enumerate(material.EPS_NAMES + material.SIG_NAMES):
        assert np.array_equal(material.fortran(got[name]), want[q]), (name, P)


def test_device_attenuation_matches_restatement():
    im, table = _case(3, ncol=3)
    got = material.attenuation_arrays_device(im, table, 4, 12.5)
    want = ref.attenuation(im, table, 4, 12.5)
    for q, name in enumerate(material.GAMMA_NAMES):
        assert np.array_equal(material.fortran(got[name]), want[q])


def test_device_pass_large_image_matches_host_pass():
    """A 1000 x 700 image with 20-cell CPML: device grids equal the host
    pass's (the host pass is itself pinned to the restatement above)."""
    im, table = _case(21, nx=1000, nz=700, nmat=9)
    got = material.stiffness_arrays_device(im, table, 20)
    want = material.stiffness_arrays(im, table, 20)
    for name in material.STIFFNESS_NAMES:
        assert np.array_equal(material.fortran(got[name]), want[name]), name


@pytest.mark.parametrize("precision", ["FP64", "FP32"])
def test_solver_from_device_material_grids(precision):
    """seismic2 on a two-material image: the stiffness pre-pass on the device
    feeds the solver's model slots directly (device to device); the run
    equals the one fed the host grids of the same pre-pass, bit for bit."""
    n, cpml, nt = 64, 10, 150
    im = np.ones((n, n), dtype=np.int32)
    im[:, n // 2:] = 2
    top, bot = models.TWO_LAYER_TOP, models.TWO_LAYER_BOTTOM
    table = np.zeros((2, 23))
    for r, lay in enumerate((top, bot)):
        table[r, 0] = r + 1
        table[r, 1] = lay["c11"]
        table[r, 3] = lay["c13"]
        table[r, 5] = lay["c15"] + 0.3e9    # c15, c35 non-zero so every slot matters
        table[r, 12] = lay["c33"]
        table[r, 14] = lay["c35"] - 0.2e9
        table[r, 19] = lay["c55"]
        table[r, 22] = lay["rho"]
    base = models.seismic2_two_layer(n=n, cpml=cpml, nt=nt, src=(n // 2, 12), nrec=16, rec_z=6)
    dev = material.stiffness_arrays_device(im, table, cpml)
    host = material.stiffness_arrays(im, table, cpml)
    keys = ("c11", "c13", "c15", "c33", "c35", "c55", "rho")
    p_host = dataclasses.replace(base, model={**base.model, **{k: host[k] for k in keys}})
    p_dev = dataclasses.replace(base, model={**base.model, **{k: dev[k] for k in keys}})
    prec = getattr(sg, precision)
    a = sg.run(p_host, prec)
    b = sg.run(p_dev, prec)
    assert np.max(np.abs(a["traces"])) > 0
    assert np.array_equal(a["traces"], b["traces"])
    for x, y in zip(a["fields"], b["fields"]):
        assert np.array_equal(x, y)


def test_device_model_grid_refused_for_em():
    import torch
    p = models.electromag2_blocks(n=32, cpml=6, nt=10, src=(16, 8), nrec=4, rec_z=4, nblocks=0)
    bad = dataclasses.replace(p, model={**p.model, "e11": torch.ones(p.nz, p.nx, dtype=torch.float64, device="cuda")})
    with pytest.raises(sg.SeidartError):
        sg.run(bad, sg.FP64)
