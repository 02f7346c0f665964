"""Argument checks of seidart_solver_create through the C ABI, made before
any device work, so they run without a GPU: each bad argument is refused
with SEIDART_ERR_ARG and a message naming it (the reference stops the
program instead, cpmlfdtd.f08 / seidartio.f08); valid arguments on a host
without a GPU are refused with SEIDART_ERR_UNSUPPORTED, never run on a CPU
fallback."""
import ctypes as C
import dataclasses

import numpy as np
import pytest
import torch

import seidart_gpu as sg
from seidart_gpu import models
from seidart_gpu._lib import SeidartError, lib, ptr_array

ARG, UNSUPPORTED = -1, -7


def _problem():
    return models.seismic2_two_layer(n=24, cpml=4, nt=10, src=(12, 6), nrec=4, rec_z=4)


def _create(p, precision=sg.FP64, density_code=None):
    model, src, rec = p.model_list(), p.src_list(), p.receiver_array()
    h = C.c_void_p()
    code = p.density_code() if density_code is None else density_code
    rc = lib().seidart_solver_create(C.byref(h), p.family, precision, C.byref(p.domain()), C.byref(p.source()), code,
                                     ptr_array(model), ptr_array(src), len(rec),
                                     rec.ctypes.data if len(rec) else None)
    if rc == 0:
        lib().seidart_solver_destroy(h)
    return rc, lib().seidart_last_error().decode()


@pytest.mark.parametrize("change,word", [
    (lambda p: dataclasses.replace(p, time_steps=0, src={}), "time_steps"),
    (lambda p: dataclasses.replace(p, dt=-1.0), "dt"),
    (lambda p: dataclasses.replace(p, dx=0.0), "spacing"),
    (lambda p: dataclasses.replace(p, xind=10_000), "source index"),
    (lambda p: dataclasses.replace(p, receivers=np.array([0, p.ncell + 5], dtype=np.int32)), "receiver"),
])
def test_bad_argument_is_refused(change, word):
    rc, msg = _create(change(_problem()))
    assert rc == ARG, (rc, msg)
    assert word in msg


def test_bad_precision_and_density_are_refused():
    p = _problem()
    rc, msg = _create(p, precision=99)
    assert rc == ARG and "precision" in msg
    rc, msg = _create(p, density_code=7)
    assert rc == ARG and "density_code" in msg


def test_valid_arguments_without_a_gpu_are_unsupported():
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(SeidartError) as e:
        sg.Solver(_problem(), sg.FP64)
    assert e.value.code == UNSUPPORTED
    assert "no CUDA device" in str(e.value)


def test_batch_arguments_are_checked_per_model():
    """seidart_batch_create: the models advance together (equal time_steps),
    and a model's own bad argument is reported with its index."""
    from seidart_gpu.batch import Batch
    probs = models.batch_layered_vti(nmodels=3, nt=10, cpml=6, nmin=24, nmax=40, step=8, nrec=4, seed=3)
    short = [probs[0], dataclasses.replace(probs[1], time_steps=5, src={k: v[:5] for k, v in probs[1].src.items()})]
    with pytest.raises(SeidartError) as e:
        Batch(short, autotune=False)
    assert e.value.code == ARG and "time_steps must match" in str(e.value)
    bad = [dataclasses.replace(probs[0], xind=10_000), probs[1]]
    with pytest.raises(SeidartError) as e:
        Batch(bad, autotune=False)
    assert e.value.code == ARG and "model 0" in str(e.value) and "source index" in str(e.value)


def test_gradient_arguments_are_checked():
    """seidart_fwi_create_family refuses a shot whose source lies outside
    the grid; the Python layer refuses families without an adjoint before
    it reaches the ABI (which would answer SEIDART_ERR_UNSUPPORTED)."""
    from seidart_gpu.fwi import Fwi, Shot
    p = _problem()
    shot = Shot(xind=12, zind=6, srcz=np.asarray(p.src["z"], dtype=np.float64))
    far = Shot(xind=10_000, zind=6, srcz=shot.srcz)
    with pytest.raises(SeidartError) as e:
        Fwi(p, [shot, far])
    assert e.value.code == ARG and "shot source outside the grid" in str(e.value)
    p3 = models.seismic3_layers(n=16, cpml=4, nt=10, nlayers=2, nrec_side=2, rec_z=2, src_z=4)
    with pytest.raises(ValueError, match="seismic2 and electromag2"):
        Fwi(p3, [Shot(xind=8, zind=4, srcz=np.asarray(p3.src["z"], dtype=np.float64))])
