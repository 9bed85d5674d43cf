"""gbmd_thermo_noalloc: the thermo reduction for callers that cannot
allocate GPU memory (a host application whose own pool owns all device
memory, or a real-time loop that must stay out of the driver's allocator).
Its partial sums sit in a fixed file-scope device array instead of memory
it would allocate.

It must return what the allocating entry point gbmd_thermo returns for the
same atoms, on two calls in a row (the second call sees the shared scratch
the first one left behind), and refuse atom counts beyond its fixed
scratch.  This file is collected last so that a failure here comes after
every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from cabanamd_gb300 import gbmd

pytestmark = pytest.mark.gpu

NOALLOC_MAX_ATOMS = 65536 * 256


def _system(n, seed):
    rng = np.random.default_rng(seed)
    L = 20.0
    x = rng.uniform(0.0, L, size=(n, 3))
    v = rng.normal(size=(n, 3))
    t = rng.integers(0, 2, size=n).astype(np.int32)
    ids = np.arange(1, n + 1, dtype=np.int32)
    return x, v, t, ids, L


def test_noalloc_thermo_matches_allocating_entry_point(gpu_ctx_factory):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    lib = gbmd.load_library()
    n = 50_000
    x, v, t, ids, L = _system(n, seed=99)
    mass = np.array([1.0, 2.5])
    mvv2e, boltz = 1.0364269e-4, 8.617343e-5  # metal units

    c = gpu_ctx_factory()
    c.set_units(boltz, mvv2e, 0.001)
    c.set_box([0, 0, 0], [L, L, L])
    c.set_types(mass)
    c.upload_atoms(x, v, t, ids)

    dev = torch.device("cuda", 0)
    v_soa = torch.tensor(np.ascontiguousarray(v.T), dtype=torch.float64, device=dev)
    t_dev = torch.tensor(t, dtype=torch.int32, device=dev)
    m_dev = torch.tensor(mass, dtype=torch.float64, device=dev)
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    for call, scale in enumerate((1.0, 2.0)):
        if scale != 1.0:
            c.scale_velocities(scale)
            v_soa.mul_(scale)
        T_ref, KE_ref = c.thermo()
        out.fill_(-1.0)
        rc = lib.gbmd_thermo_noalloc(v_soa.data_ptr(), t_dev.data_ptr(), m_dev.data_ptr(), n,
                                     mvv2e, boltz, C.c_void_p(stream.cuda_stream),
                                     out.data_ptr())
        assert rc == gbmd.GBMD_OK, f"call {call}: rc={rc}"
        stream.synchronize()
        T, KE = out.cpu().tolist()
        assert np.isclose(T, T_ref, rtol=1e-10, atol=0), (call, T, T_ref)
        assert np.isclose(KE, KE_ref, rtol=1e-10, atol=0), (call, KE, KE_ref)
    c.close()


def test_noalloc_thermo_rejects_oversize_and_bad_args(gpu_ctx_factory):
    torch = pytest.importorskip("torch")
    lib = gbmd.load_library()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(8, dtype=torch.float64, device=dev)
    ti = torch.zeros(8, dtype=torch.int32, device=dev)
    p = buf.data_ptr()
    # beyond the fixed scratch: a clear capacity error, nothing launched
    assert lib.gbmd_thermo_noalloc(p, ti.data_ptr(), p, NOALLOC_MAX_ATOMS + 1, 1.0, 1.0, None,
                                   p) == 3
    assert lib.gbmd_thermo_noalloc(None, ti.data_ptr(), p, 8, 1.0, 1.0, None, p) == 1
    assert lib.gbmd_thermo_noalloc(p, ti.data_ptr(), p, 1, 1.0, 1.0, None, p) == 1
