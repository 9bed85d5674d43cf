"""Host <-> device transfers of the atom arrays (gbmd_upload_atoms,
gbmd_download_atoms; System::resize + deep_copy, inputFile_impl.h:791,849,865).

Arrays registered with gbmd_host_register are read and written in place by
kernels over the host link; other arrays go through staged copies.  Both
paths must move exactly the same bytes, and an array only partly inside a
registered range must never be read through the mapping."""
import numpy as np
import pytest

from cabanamd_gb300 import inputs


def _pinned_copy(a):
    from cabanamd_gb300 import gbmd
    out = gbmd.aligned_empty(a.shape, a.dtype)
    out[...] = a
    return out


def _ctx(factory, st):
    c = factory()
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.lj_coeff(1, 1, 1.0, 1.0, 2.5)
    return c


def _run(c, st, x, v, t, i, out):
    c.upload_atoms(x, v, t, i)
    c.exchange()
    c.binning(2.8)
    c.neigh_build(2.8, 0, 96)
    c.zero_force()
    c.force_compute()
    return c.download_atoms(out)


def _same(a, b):
    for k in ("x", "v", "f", "type", "id"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k


@pytest.mark.gpu
def test_registered_arrays_move_the_same_bytes(gpu_ctx_factory):
    """Upload from and download into registered arrays (the direct kernels)
    against plain arrays (the copy path): identical x, v, f, type and id,
    at an atom count that is not a multiple of the 256-atom transfer block."""
    from cabanamd_gb300 import gbmd
    st = inputs.lj_fcc(26, T=1.44, seed=91)  # 70,304 atoms
    st.x = st.x[:70001]
    st.v = st.v[:70001]
    st.type = st.type[:70001]
    st.id = st.id[:70001]
    n = len(st.x)
    assert n % 256 != 0
    c = _ctx(gpu_ctx_factory, st)
    plain = _run(c, st, st.x, st.v, st.type, st.id, None)
    px, pv, pt, pi = (_pinned_copy(a) for a in (st.x, st.v, st.type.astype(np.int32),
                                                st.id.astype(np.int32)))
    out = gbmd.Atoms(gbmd.aligned_empty((n, 3), np.float64), gbmd.aligned_empty((n, 3), np.float64),
                     gbmd.aligned_empty((n, 3), np.float64), gbmd.aligned_empty(n, np.int32),
                     gbmd.aligned_empty(n, np.int32))
    with gbmd.PinnedHost(px, pv, pt, pi, out.x, out.v, out.f, out.type, out.id):
        direct = _run(c, st, px, pv, pt, pi, out)
        _same(plain, direct)
        # registered upload, plain download and the reverse
        _same(plain, _run(c, st, px, pv, pt, pi, None))
        _same(plain, _run(c, st, st.x, st.v, st.type, st.id, out))
        # a NULL array is skipped by the direct download
        out.v[...] = -7.0
        lib = c.lib
        rc = lib.gbmd_download_atoms(c.h, out.x.ctypes.data, None, out.f.ctypes.data,
                                     out.type.ctypes.data, None)
        assert rc == 0
        assert np.all(out.v == -7.0)
        assert np.array_equal(out.x, plain.x) and np.array_equal(out.f, plain.f)
    c.close()


@pytest.mark.gpu
def test_registered_upload_without_velocities_and_bad_types(gpu_ctx_factory):
    """v = NULL through the direct kernel gives zero velocities; a type out
    of range is still an error that leaves no atoms."""
    from cabanamd_gb300 import gbmd
    st = inputs.lj_fcc(6, T=1.44, seed=3)
    n = len(st.x)
    px = _pinned_copy(st.x)
    pt = _pinned_copy(st.type.astype(np.int32))
    pi = _pinned_copy(st.id.astype(np.int32))
    c = _ctx(gpu_ctx_factory, st)
    with gbmd.PinnedHost(px, pt, pi):
        c.upload_atoms(px, None, pt, pi)
        a = c.download_atoms()
        assert np.all(a.v == 0.0)
        assert np.array_equal(np.sort(a.id), np.sort(st.id))
        pt[n // 2] = 5
        with pytest.raises(gbmd.GbmdError):
            c.upload_atoms(px, None, pt, pi)
        assert c.num_atoms() == 0
    c.close()


@pytest.mark.gpu
def test_array_partly_inside_a_registered_range_is_not_read_through_the_mapping(gpu_ctx_factory):
    """Only the first half of the position array is registered.  The upload
    must not take the direct kernel (it would read past the mapping); the copy
    path then meets CUDA's refusal to copy from a partly pinned range, which
    comes back as an error.  Either way the context stays usable: a plain
    upload afterwards gives the plain result."""
    from cabanamd_gb300 import gbmd
    st = inputs.lj_fcc(8, T=1.44, seed=4)
    px = _pinned_copy(st.x)
    c = _ctx(gpu_ctx_factory, st)
    plain = _run(c, st, st.x, st.v, st.type, st.id, None)
    lib = gbmd.load_library()
    half = (px.nbytes // 2) & ~4095
    assert lib.gbmd_host_register(px.ctypes.data, half) == 0
    try:
        got = _run(c, st, px, st.v, st.type, st.id, None)
        _same(plain, got)
    except gbmd.GbmdError as err:
        assert err.code == 2  # GBMD_ERR_CUDA
    finally:
        lib.gbmd_host_unregister(px.ctypes.data)
    _same(plain, _run(c, st, st.x, st.v, st.type, st.id, None))
    c.close()
