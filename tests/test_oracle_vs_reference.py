"""The oracle restatement against the reference's own CPU kernel (kernels/cpu built from the reference
sources by oracle/ref_build.py): forces and energies of the same FP64 positions agree to rounding, and
ensembles of A + B <-> C runs agree in their mean counts within 3 sigma.  Skipped where the reference
sources are absent (the library is built from the reference tree or its staged copy)."""
import concurrent.futures as cf

import numpy as np
import pytest

import oracle
from oracle import reference_kernel as rk
from tests.helpers import abc_spec, crowded_spec, f32, make_oracle

pytestmark = pytest.mark.skipif(not rk.available(), reason="reference CPU kernel cannot be built here")


def _reference(spec, n_threads=4):
    k = rk.ReferenceKernel(spec["box"], spec.get("periodic", (True, True, True)), 1.0, spec["diffusion"], n_threads)
    for kind, a, b, p in spec.get("potentials", []):
        if kind == "harmonic_repulsion":
            k.add_harmonic_repulsion(a, b, p["k"], p["d"])
        elif kind == "weak_interaction_piecewise_harmonic":
            k.add_weak_interaction_piecewise_harmonic(a, b, p["k"], p["desired"], p["depth"], p["cutoff"])
        elif kind == "lennard_jones":
            k.add_lennard_jones(a, b, p["m"], p["n"], p["cutoff"], p["shift"], p["epsilon"], p["sigma"])
    for kind, p in spec.get("reactions", []):
        if kind == "fusion":
            k.add_fusion(p["a"], p["b"], p["c"], p["rate"], p["educt_distance"])
        elif kind == "fission":
            k.add_fission(p["a"], p["b"], p["c"], p["rate"], p["product_distance"])
    return k


@pytest.mark.parametrize("system", ["abc", "crowded"])
def test_oracle_forces_equal_the_reference_kernel(system):
    """Forces and energy of the oracle and of the reference's CalculateForces on identical positions."""
    if system == "abc":
        spec, pos, types = abc_spec(n=4000, box=25.0, seed=3)
    else:
        spec, pos, types = crowded_spec(n=20000, density=0.2, seed=4)
    spec["reactions"] = []
    pos = f32(pos)
    ref = _reference(spec)
    ref.add_particles(pos, types)
    ids, f_ref, e_ref = ref.calculate_forces(len(pos))
    f_ref = f_ref[np.argsort(ids)]
    o = make_oracle(spec, n_threads=4)
    o.add_particles(pos, types)
    o.nl_setup(o.calculate_max_cutoff())
    e = o.calculate_forces()
    _, _, oid, f, _ = o.particles()
    f = f[np.argsort(oid)]
    scale = np.abs(f_ref).max()
    assert np.abs(f - f_ref).max() <= 1e-12 * scale
    assert abs(e - e_ref) <= 1e-12 * abs(e_ref)


@pytest.mark.parametrize("handler", [oracle.UNCONTROLLED_APPROXIMATION, oracle.GILLESPIE])
def test_oracle_ensemble_matches_the_reference_kernel_ensemble(handler):
    """24 runs each of 100 A + 100 B in a 10^3 box, 2000 steps of 5e-3: the mean final counts agree within
    3 sigma (the random streams differ, so the comparison is statistical)."""
    spec, pos, types = abc_spec(n=200, box=10.0, seed=1)
    pos = f32(pos)
    n_runs = 24

    def ref_run(r):
        k = _reference(spec, n_threads=1)
        k.add_particles(pos, types)
        return k.run(2000, 5e-3, handler=handler)[0][2]

    def orc_run(r):
        o = make_oracle(spec, seed=700 + r)
        o.add_particles(pos, types)
        return o.run(2000, 5e-3, handler=handler, count_stride=2000)[-1, 2]

    with cf.ThreadPoolExecutor(8) as ex:
        a = np.array(list(ex.map(ref_run, range(n_runs))), float)
        b = np.array(list(ex.map(orc_run, range(n_runs))), float)
    sigma = np.sqrt(a.var(ddof=1) / n_runs + b.var(ddof=1) / n_runs)
    assert abs(a.mean() - b.mean()) <= 3 * sigma, (a.mean(), b.mean(), sigma)
