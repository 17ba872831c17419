"""esm_capacity_scores_static (the score entry point that allocates nothing in the call) against
esm_capacity_scores on the same state, through the C ABI, on two calls in a row; a first call with
no other device work before it leaves the device's free memory unchanged; and its size limit.
Collected last so that it also runs after every other GPU test."""
import numpy as np
import pytest

from esmgb.device import DeviceChain, EsmError
from esmgb.model import initial_state, make_model

pytestmark = pytest.mark.gpu


def _state(m, R, seed=3):
    st = initial_state(m, R, seed=seed)
    rng = np.random.Generator(np.random.PCG64(seed))
    st.g = st.g + 0.05 * rng.standard_normal(st.g.shape)
    st.e = rng.uniform(0.05, 0.95, st.e.shape)
    return st


@pytest.mark.parametrize("prec", [64, 32])
def test_static_scores_match(prec):
    m = make_model(40, 60, 40, seed=11)
    st = _state(m, 32)
    d = DeviceChain(m, 32, precision=prec, seed=5)
    d.upload(st)
    d.sweeps(1, 0)
    sk0, fk0, p0 = d.scores()
    scale = np.abs(sk0).max(axis=0) + 1e-3
    for _ in range(2):                     # two calls in a row: the scratch is cleared each time
        sk, fk, parts = d.scores_static()
        # the score sums are FP64 atomics in both entry points: equal up to summation order
        assert (np.abs(sk - sk0) / scale).max() < 1e-9
        np.testing.assert_allclose(fk, fk0, rtol=1e-14)
        np.testing.assert_allclose(parts, p0, rtol=1e-9, atol=1e-6)
    d.close()


def _free_device_bytes():
    """Free device memory (cudaMemGetInfo) through the CUDA runtime loaded in this process, else the
    toolkit's; None when neither can be found."""
    import ctypes
    import os
    paths = [ln.split()[-1] for ln in open("/proc/self/maps") if "libcudart" in ln]
    paths += ["/usr/local/cuda/lib64/libcudart.so"]
    for path in paths:
        if os.path.exists(path):
            rt = ctypes.CDLL(path)
            free, total = ctypes.c_size_t(), ctypes.c_size_t()
            if rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0:
                return free.value
    return None


@pytest.mark.parametrize("prec", [64, 32])
def test_static_scores_first_call_allocates_nothing(prec):
    """A context whose first device work after the upload is the static scores: the device's free
    memory is the same before and after the call (esm_create resolved the scratch array and loaded
    the score kernels), and the scores equal esm_capacity_scores'."""
    m = make_model(40, 60, 40, seed=13)
    d = DeviceChain(m, 16, precision=prec, seed=7)
    d.upload(_state(m, 16, seed=5))
    d.sync(60.0)
    free0 = _free_device_bytes()
    if free0 is None:
        pytest.skip("no CUDA runtime to read the free device memory")
    sk, fk, parts = d.scores_static()
    free1 = _free_device_bytes()
    assert free1 == free0, f"the call placed {free0 - free1} bytes on the device"
    sk0, fk0, p0 = d.scores()
    scale = np.abs(sk0).max(axis=0) + 1e-3
    assert (np.abs(sk - sk0) / scale).max() < 1e-9
    np.testing.assert_allclose(fk, fk0, rtol=1e-14)
    d.close()


def test_static_scores_size_limit():
    m = make_model(40, 60, 2, seed=11)
    R = (1 << 19) // (m.Kunits + 8) + 1    # one replica beyond the static scratch (2 R (K + 8) sums)
    d = DeviceChain(m, R, precision=64, seed=5)
    d.upload(_state(m, R))
    with pytest.raises(EsmError, match="static scratch holds"):
        d.scores_static()
    d.close()
