"""rdc_forces_noalloc: forces of caller-owned device arrays with the library's static scratch, for
callers that cannot let the library call cudaMalloc (embeddings whose own pool owns the GPU's memory).

Compared with the allocating entry point (rdc_calculate_forces + rdc_get_forces on a system holding
the same particles) and with the FP64 oracle on two calls in a row, so the second call checks that
nothing left in the scratch by the first changes the result.  The file is named to be collected after
every other test file: it must pass after the rest of the suite has run in the same process as well as
alone.
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

    o = make_oracle(spec, n_threads=8)
    o.add_particles(pos, types)
    o.nl_setup(o.calculate_max_cutoff())
    e_orc = o.calculate_forces()
    _, _, o_ids, f_orc, _ = o.particles()
    scale = o.force_scales()[np.argsort(o_ids)]
    f_orc = f_orc[np.argsort(o_ids)]

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
        assert np.isfinite(f).all(), f"call {call}: forces not written for every particle"
        for ref, e_ref, what in ((f_sys, e_sys, "allocating path"), (f_orc, e_orc, "oracle")):
            err = _force_err(f, ref, scale)
            assert err.max() <= FORCE_RTOL, f"call {call}: max relative force difference to the {what} {err.max():.3e}"
            assert abs(e - e_ref) <= ENERGY_RTOL * abs(e_ref), f"call {call}: energy {e} vs {e_ref} ({what})"


def _force_err(f, ref, scale):
    fn = np.linalg.norm(ref, axis=1)
    denom = np.maximum(fn, FLOOR * scale)
    denom = np.where(denom > 0, denom, 1.0)
    return np.linalg.norm(f - ref, axis=1) / denom


def _noalloc(lib, torch, ctx, pos, types):
    """One call on device copies of pos/types; returns (forces, energy) on the host."""
    dev = torch.device("cuda:0")
    p_d = torch.as_tensor(np.asarray(pos, np.float32), device=dev).contiguous()
    t_d = torch.as_tensor(np.asarray(types, np.int32), device=dev).contiguous()
    f_d = torch.full((len(pos), 3), float("nan"), dtype=torch.float32, device=dev)
    e_d = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = lib.rdc_forces_noalloc(ctx.handle, len(pos), p_d.data_ptr(), t_d.data_ptr(), f_d.data_ptr(),
                                e_d.data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
    assert rc == 0, lib.rdc_last_error().decode()
    torch.cuda.synchronize()
    return f_d.cpu().numpy().astype(np.float64), float(e_d.cpu().item())


def _oracle(spec, pos, types):
    o = make_oracle(spec, n_threads=8)
    o.add_particles(pos, types)
    o.nl_setup(o.calculate_max_cutoff())
    e = o.calculate_forces()
    _, _, ids, f, _ = o.particles()
    order = np.argsort(ids)
    return f[order], o.force_scales()[order], e


@pytest.mark.gpu
def test_noalloc_alternating_contexts_and_a_widened_grid():
    """Calls for two contexts in turn re-copy the potential tables each time and give each context's
    forces; the second context's box (small cutoff, large box) needs more cells than the scratch holds,
    so its grid is widened.  Both against the oracle."""
    torch = pytest.importorskip("torch")
    lib = _lib()
    spec_a, pos_a, types_a = crowded_spec(n=20000, density=0.2, seed=12)
    rng = np.random.default_rng(5)
    L = 80.0  # 80^3 cells at the cutoff of 1.0: widened to fit 131072 cells
    pos_b = f32((rng.random((30000, 3)) - 0.5) * L)
    types_b = rng.integers(0, 2, len(pos_b)).astype(np.int32)
    spec_b = dict(box=(L, L, L), periodic=(True, True, True), diffusion=(1.0, 1.0),
                  potentials=[("harmonic_repulsion", a, b, dict(k=10.0, d=1.0)) for a, b in [(0, 0), (0, 1), (1, 1)]])
    cases = [(make_context(spec_a), spec_a, f32(pos_a), types_a), (make_context(spec_b), spec_b, pos_b, types_b)]
    refs = [_oracle(spec, pos, types) for _, spec, pos, types in cases]
    for rnd in range(2):
        for (ctx, _, pos, types), (f_ref, scale, e_ref) in zip(cases, refs):
            f, e = _noalloc(lib, torch, ctx, pos, types)
            err = _force_err(f, f_ref, scale)
            assert err.max() <= FORCE_RTOL, (rnd, err.max())
            assert abs(e - e_ref) <= ENERGY_RTOL * abs(e_ref), (rnd, e, e_ref)


@pytest.mark.gpu
def test_noalloc_bad_type_or_position_makes_the_energy_nan():
    """A type outside the context's species, a NaN coordinate or a coordinate outside the box on a
    periodic axis: that particle gets no force and the energy is NaN; the next clean call is clean."""
    torch = pytest.importorskip("torch")
    lib = _lib()
    spec, pos, types = crowded_spec(n=5000, density=0.2, seed=13)
    pos, types = f32(pos), np.asarray(types, np.int32)
    ctx = make_context(spec)
    L = spec["box"][0]
    for what in ("type", "nan", "outside"):
        p, t = pos.copy(), types.copy()
        if what == "type":
            t[17] = -1
        elif what == "nan":
            p[17, 1] = np.nan
        else:
            p[17, 2] = 0.75 * L
        f, e = _noalloc(lib, torch, ctx, p, t)
        assert np.isnan(e), what
        assert np.all(f[17] == 0.0), (what, f[17])
    f, e = _noalloc(lib, torch, ctx, pos, types)
    assert np.isfinite(e) and np.isfinite(f).all()
