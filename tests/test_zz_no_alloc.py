"""seidart_trace_misfit_noalloc: the trace misfit with its scratch in a fixed
device array, against the misfit seidart_fwi_gradient computes on the same
traces (FP32 residuals, FP64 sums; equal up to summation order).  Two calls
in a row must both agree, so the scratch is cleared between calls.  This
file is named to be collected last; it passes alone as well.
"""
import ctypes as C

import numpy as np
import pytest

REL = 1e-12  # FP64 sums of the same FP32 residuals in another order


def _fn():
    from seidart_gpu._lib import lib
    f = lib().seidart_trace_misfit_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    return f


def _last_error():
    from seidart_gpu._lib import lib
    return lib().seidart_last_error().decode()


@pytest.mark.gpu
def test_noalloc_misfit_matches_fwi_misfit_twice():
    torch = pytest.importorskip("torch")
    from seidart_gpu import models
    from seidart_gpu.fwi import Fwi, Shot
    p = models.seismic2_two_layer(n=64, cpml=10, nt=200, nrec=24, rec_z=6)
    shots = [Shot(20, 8, p.src["z"]), Shot(44, 8, p.src["z"])]
    with Fwi(p, shots) as f:
        syn = f.model_traces()  # [nshots][nt][2][nrec], FP32 values
    rng = np.random.default_rng(5)
    obs = syn * (1.0 + 0.05 * rng.standard_normal(syn.shape)) + 1e-7 * rng.standard_normal(syn.shape)
    with Fwi(p, shots, list(obs)) as f:
        ref = f.loss()
    syn32, obs32 = syn.astype(np.float32), obs.astype(np.float32)
    res32 = syn32 - obs32
    ntr = 2 * len(p.receivers)
    fn = _fn()
    stream = torch.cuda.Stream()
    d_syn = torch.tensor(syn32, device="cuda")
    d_obs = torch.tensor(obs32, device="cuda")
    d_res = torch.zeros_like(d_syn)
    torch.cuda.synchronize()
    for call in range(2):
        total = 0.0
        per = np.zeros((len(shots), ntr))
        for s in range(len(shots)):
            t = C.c_double()
            rc = fn(d_syn[s].data_ptr(), d_obs[s].data_ptr(), d_res[s].data_ptr(), p.time_steps, ntr,
                    per[s].ctypes.data, C.byref(t), stream.cuda_stream)
            assert rc == 0, _last_error()
            total += t.value
            assert t.value == pytest.approx(per[s].sum(), rel=REL, abs=0.0)
        assert total == pytest.approx(ref, rel=REL, abs=0.0), call
        want = 0.5 * (res32.astype(np.float64) ** 2).reshape(len(shots), p.time_steps, ntr).sum(axis=1)
        np.testing.assert_allclose(per, want, rtol=REL, atol=0.0)
        assert np.array_equal(d_res.cpu().numpy(), res32)


@pytest.mark.gpu
def test_noalloc_misfit_rejects_too_many_traces():
    torch = pytest.importorskip("torch")
    fn = _fn()
    x = torch.zeros(8193, device="cuda")
    t = C.c_double()
    rc = fn(x.data_ptr(), x.data_ptr(), None, 1, 8193, None, C.byref(t), None)
    assert rc == -1
    assert "SEIDART_NOALLOC_MAX_TRACES" in _last_error()
