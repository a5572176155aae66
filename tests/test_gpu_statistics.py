"""Statistical parity of the stochastic path.  The random streams differ from the reference's, so
trajectories are compared through observables: the time-averaged substrate count of the reference's
Michaelis-Menten integration test, and the ensemble distribution of species counts and reaction counts
of A + B <-> C against an ensemble of oracle runs (within 3 sigma)."""
import numpy as np
import pytest

import oracle
from tests.golden import known_answers as ka
from tests.helpers import abc_spec, make_context, make_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rg():
    import readdy_gb300
    readdy_gb300.load()
    return readdy_gb300


def michaelis_menten_system(rg, seed):
    mm = ka.MICHAELIS_MENTEN
    ctx = rg.Context(mm["box"], mm["periodic"], 1.0, mm["diffusion"])
    ctx.add_fusion(0, 1, 2, mm["k_fwd"], mm["educt_distance"])      # E + S -> ES
    ctx.add_fission(2, 0, 1, mm["k_back"], mm["product_distance"])  # ES -> E + S
    ctx.add_fission(2, 0, 3, mm["k_prod"], mm["product_distance"])  # ES -> E + P
    rng = np.random.default_rng(seed)
    L = mm["box"][0]
    n = mm["n_e"] + mm["n_s"]
    pos = (rng.random((n, 3)) - 0.5) * L
    types = np.array([0] * mm["n_e"] + [1] * mm["n_s"])
    k = rg.CUDAKernel(ctx, seed=seed)
    k.add_particles(pos, types)
    return k


@pytest.mark.parametrize("handler", ["uncontrolled_approximation", "gillespie"])
def test_michaelis_menten_time_averaged_substrate(rg, handler):
    """readdy/test/IntegrationTests.cpp:30-106: 70 E + 700 S, 37500 steps of 8e-3; the substrate count
    averaged over all 37501 observations lies within 3 % of 665.2."""
    mm = ka.MICHAELIS_MENTEN
    h = rg.GILLESPIE if handler == "gillespie" else rg.UNCONTROLLED_APPROXIMATION
    k = michaelis_menten_system(rg, seed=2024)
    counts = k.run(mm["n_steps"], mm["dt"], handler=h, count_stride=1)
    assert counts.shape == (mm["n_steps"] + 1, 4)
    assert np.all(counts[:, 0] + counts[:, 2] == mm["n_e"])                 # enzyme conserved
    assert np.all(counts[:, 1] + counts[:, 2] + counts[:, 3] == mm["n_s"])  # substrate conserved
    mean_s = counts[:, 1].mean()
    assert abs(mean_s - mm["mean_s"]) < mm["rel_band"] * mm["mean_s"], mean_s


@pytest.mark.parametrize("handler", ["uncontrolled_approximation", "gillespie"])
def test_counts_and_reaction_rates_match_an_oracle_ensemble(rg, handler):
    """100 A + 100 B in a 10^3 box with harmonic repulsion, A + B -> C (k = 1) and C -> A + B (k = 0.1),
    2000 steps of 5e-3 from one initial configuration: the ensemble means of the final C count and of the
    fusion and fission counts agree between 48 GPU runs and 48 oracle runs within 3 sigma."""
    spec, pos, types = abc_spec(n=200, box=10.0, seed=1)
    h_gpu = rg.GILLESPIE if handler == "gillespie" else rg.UNCONTROLLED_APPROXIMATION
    h_orc = oracle.GILLESPIE if handler == "gillespie" else oracle.UNCONTROLLED_APPROXIMATION
    n_runs, n_steps, dt = 48, 2000, 5e-3
    gpu, orc = [], []
    for r in range(n_runs):
        k = rg.CUDAKernel(make_context(spec), seed=1000 + r)
        k.add_particles(pos, types)
        c = k.run(n_steps, dt, handler=h_gpu, count_stride=n_steps)
        gpu.append([c[-1, 2], *k.reaction_counts()[:2]])
        o = make_oracle(spec, seed=5000 + r)
        o.add_particles(pos, types)
        c = o.run(n_steps, dt, handler=h_orc, count_stride=n_steps)
        orc.append([c[-1, 2], *o.reaction_counts(2)])
    gpu, orc = np.array(gpu, float), np.array(orc, float)
    for q, name in enumerate(["final C", "fusions", "fissions"]):
        diff = gpu[:, q].mean() - orc[:, q].mean()
        sigma = np.sqrt(gpu[:, q].var(ddof=1) / n_runs + orc[:, q].var(ddof=1) / n_runs)
        assert abs(diff) <= 3 * sigma, f"{name}: GPU {gpu[:, q].mean():.2f} vs oracle {orc[:, q].mean():.2f} (sigma {sigma:.2f})"
