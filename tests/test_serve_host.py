"""Host side of the served form: the seeded request stream and the admission arithmetic (no GPU)."""
import numpy as np
import pytest

from readdy_gb300.serve import Server, reaction_network, serving_workload


def test_stream_is_seeded_and_within_its_ranges():
    a = serving_workload(seed=3, n_requests=300)
    b = serving_workload(seed=3, n_requests=300)
    assert [s.n_steps for s in a] == [s.n_steps for s in b]
    assert all(np.array_equal(x.positions, y.positions) for x, y in zip(a[:5], b[:5]))
    arr = np.array([s.arrival for s in a])
    assert np.all(np.diff(arr) > 0)
    assert abs(np.mean(np.diff(arr)) - 1 / 20.0) < 0.15 / 20.0 * 3  # Poisson arrivals at 20 per second
    for s in a:
        n = len(s.positions)
        assert 2 <= s.n_types <= 6 and 500 <= n <= 200000
        assert 0.1 <= n / s.box ** 3 <= 0.5 + 1e-6
        assert 1000 <= s.n_steps <= 100000
        assert all(0.1 <= d <= 2.0 for d in s.diffusion)
        assert np.all(np.abs(s.positions) <= s.box / 2)
        for kind, args in s.reactions:
            rate = args[3] if kind in ("fusion", "fission") else args[2]
            assert 1e-3 <= rate <= 1.0


@pytest.mark.parametrize("seed", range(20))
def test_reaction_network_conserves_mass(seed):
    rng = np.random.default_rng(seed)
    T = 2 + seed % 5
    reactions, mass = reaction_network(rng, T)
    assert mass[0] == 1 and len(mass) == T
    for kind, args in reactions:
        if kind == "fusion":
            i, j, k = args[:3]
            assert mass[i] + mass[j] == mass[k]
        elif kind == "fission":
            k, i, j = args[:3]
            assert mass[k] == mass[i] + mass[j]
        else:
            i, k = args[:2]
            assert mass[i] == mass[k]


def test_request_bytes_choose_the_leg_and_grow_with_the_request():
    s = serving_workload(seed=1, n_requests=1)[0]
    ctx = s.context()
    small, p_small = Server.request_bytes(ctx, 1000, 1000, 100, plain_threshold=32768)
    big, p_big = Server.request_bytes(ctx, 100000, 1000, 100, plain_threshold=32768)
    assert not p_small and p_big
    assert small < big
    b1, _ = Server.request_bytes(ctx, 5000, 1000, 100)
    b2, _ = Server.request_bytes(ctx, 5000, 100000, 100)
    assert b2 > b1  # the count records are part of the footprint
    # particle state: two float4 buffers, two id buffers and five int scratch arrays per slot
    assert b1 >= (5000 + 5000 // 4 + 64) * (32 + 8 + 20)
