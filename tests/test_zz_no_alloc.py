"""eprem_gpu_omni_flux_static -- the flux entry point that allocates nothing
-- against eprem_gpu_omni_flux, called through the C ABI.  Collected last so
that it also runs after every other GPU test has used the device; it must
pass on its own as well.

Both entry points run the same flux kernel, so the values agree exactly; the
check allows a relative 1e-12, the FP64 parity tolerance of this suite."""
import ctypes as C

import numpy as np
import pytest

from eprem_gb300 import EpremRun, abi, workloads as W
from eprem_gb300.runtime import EpremGpuError
from helpers import primed_state

pytestmark = pytest.mark.gpu

DP = C.POINTER(C.c_double)


def _flux(run, fn):
    d = run.dims
    out = np.full(d.num_streams * d.num_nodes * d.num_energies, np.nan)
    rc = fn(run.handle, out.ctypes.data_as(DP))
    assert rc == 0, run.lib.eprem_gpu_last_error().decode()
    return out


def _close(a, b):
    assert np.all(np.isfinite(a)) and np.all(np.isfinite(b))
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=0.0)


def test_static_flux_matches_allocating_flux_twice(oracle_lib):
    w = W.custom(1, 1, 120, 8, 10, num_ep_steps=3)
    d, g, f, nodes = primed_state(w, oracle_lib)
    run = EpremRun(d, w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    run.update_energetic_particles(0.0)
    static = run.lib.eprem_gpu_omni_flux_static
    first = _flux(run, static)
    second = _flux(run, static)
    plain = _flux(run, run.lib.eprem_gpu_omni_flux)
    _close(first, plain)
    _close(second, plain)
    # the buffer holds stale values from the call before; a new state must
    # still come out whole
    run.update_energetic_particles(w.params.t_del)
    third = _flux(run, static)
    _close(third, _flux(run, run.lib.eprem_gpu_omni_flux))
    assert np.max(np.abs(third - first)) > 0.0
    run.close()


def test_static_flux_allocates_no_device_memory(oracle_lib):
    """Free device memory is the same before the first static call on a
    fresh run and after three of them: the buffer is resident from the run's
    creation on, and the call allocates nothing (the kernel's own module was
    loaded by the run's earlier update)."""
    torch = pytest.importorskip("torch")
    w = W.custom(1, 1, 60, 6, 8, num_ep_steps=1)
    d, g, f, nodes = primed_state(w, oracle_lib)
    run = EpremRun(d, w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    run.update_energetic_particles(0.0)
    run.omni_flux()  # loads the flux kernel's module; allocates the plain entry's buffer
    run.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    out = run.omni_flux_static()
    again = [run.omni_flux_static() for _ in range(2)]
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0
    for a in again:
        _close(a, out)
    run.close()


def test_static_flux_rejects_sizes_beyond_its_buffer():
    # 96 streams x 1000 nodes x 11 energies = 1,056,000 > 1,048,576
    w = W.custom(4, 4, 1000, 11, 4, num_ep_steps=1)
    d = w.dims()
    assert d.num_streams * d.num_nodes * d.num_energies > abi.FLUX_STATIC_MAX
    run = EpremRun(d, w.params, W.build_grids(w))
    with pytest.raises(EpremGpuError) as e:
        run.omni_flux_static()
    assert e.value.code == abi.EPREM_GPU_ERR_ARG
    assert "exceed the static buffer" in str(e.value)
    run.close()
