"""rdc_forces_noalloc: forces of caller-owned device arrays with the library's static scratch.

Compared with the allocating entry point (rdc_calculate_forces + rdc_get_forces on a system holding
the same particles) on two calls in a row, so the second call checks that nothing left in the scratch
by the first changes the result.  The file is named to be collected after every other test file: it
must pass after the rest of the suite has run in the same process as well as alone.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import crowded_spec, f32, make_context, make_oracle

FORCE_RTOL = 1e-5   # |dF| <= FORCE_RTOL * max(|F|, FLOOR * S), S = sum of |term| of the particle
FLOOR = 0.1
ENERGY_RTOL = 1e-5


def _lib():
    from readdy_gb300 import _native
    return _native.load()


def test_rejects_more_particles_than_the_scratch_holds():
    """Host-side limit check: fails before any device work, so it needs no GPU."""
    import readdy_gb300 as rg
    lib = _lib()
    ctx = rg.Context((10.0, 10.0, 10.0), diffusion_constants=(1.0,))
    ctx.add_harmonic_repulsion(0, 0, 10.0, 1.0)
    dummy = (C.c_float * 4)()
    energy = C.c_double()
    n = 65536 + 1
    rc = lib.rdc_forces_noalloc(ctx.handle, n, C.addressof(dummy), C.addressof(dummy), C.addressof(dummy),
                                C.addressof(energy), None)
    assert rc == 1  # RDC_ERR_INVALID_ARGUMENT
    msg = lib.rdc_last_error().decode()
    assert "65537 particles exceed the scratch limit of 65536" in msg
    assert lib.rdc_forces_noalloc(ctx.handle, -1, None, None, None, C.addressof(energy), None) == 1


@pytest.mark.gpu
def test_noalloc_forces_match_the_allocating_path_twice():
    torch = pytest.importorskip("torch")
    import readdy_gb300 as rg
    lib = _lib()
    spec, pos, types = crowded_spec(n=20000, density=0.2, seed=11)
    pos = f32(pos)
    ctx = make_context(spec)

    # allocating path: a system holding the particles, ids 0..n-1 in insertion order
    k = rg.CUDAKernel(ctx, seed=1)
    k.add_particles(pos, types)
    k.create_neighbor_list(ctx.calculate_max_cutoff())
    k.calculate_forces()
    f_sys, ids = k.get_forces()
    order = np.argsort(ids)
    f_sys = f_sys[order]
    e_sys = k.energy

    o = make_oracle(spec)
    o.add_particles(pos, types)
    o.nl_setup(o.calculate_max_cutoff())
    o.calculate_forces()
    _, _, o_ids, _, _ = o.particles()
    scale = o.force_scales()[np.argsort(o_ids)]

    dev = torch.device("cuda:0")
    p_d = torch.as_tensor(pos.astype(np.float32), device=dev).contiguous()
    t_d = torch.as_tensor(np.asarray(types, np.int32), device=dev).contiguous()
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        f_d = torch.full((len(pos), 3), float("nan"), dtype=torch.float32, device=dev)
        e_d = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = lib.rdc_forces_noalloc(ctx.handle, len(pos), p_d.data_ptr(), t_d.data_ptr(), f_d.data_ptr(),
                                    e_d.data_ptr(), stream.cuda_stream)
        assert rc == 0, lib.rdc_last_error().decode()
        torch.cuda.synchronize()
        f = f_d.cpu().numpy().astype(np.float64)
        e = float(e_d.cpu().item())
        fn = np.linalg.norm(f_sys, axis=1)
        denom = np.maximum(fn, FLOOR * scale)
        denom = np.where(denom > 0, denom, 1.0)
        err = np.linalg.norm(f - f_sys, axis=1) / denom
        assert np.isfinite(f).all(), f"call {call}: forces not written for every particle"
        assert err.max() <= FORCE_RTOL, f"call {call}: max relative force difference {err.max():.3e}"
        assert abs(e - e_sys) <= ENERGY_RTOL * abs(e_sys), f"call {call}: energy {e} vs {e_sys}"
