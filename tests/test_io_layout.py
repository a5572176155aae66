"""ReaDDy's observable file layout written as arrays (readdy_gb300/io.py): dataset paths, element types
and the flat-trajectory limits, through a save/load round trip."""
import numpy as np

from readdy_gb300 import io


def test_n_particles_and_flat_trajectory_layouts_round_trip(tmp_path):
    steps = [0, 100, 200]
    counts = np.array([[5, 3], [4, 4], [2, 6]])
    rng = np.random.default_rng(0)
    frames = [(rng.random((n, 3)), rng.integers(0, 2, n), np.arange(n) + 10 * k) for k, n in enumerate([4, 6, 5])]
    path = tmp_path / "obs.npz"
    io.save_layout(str(path), io.n_particles_layout(steps, counts), io.flat_trajectory_layout(frames, steps))
    got = io.load_layout(str(path))
    assert got["readdy/observables/n_particles/data"].dtype == np.uint64
    np.testing.assert_array_equal(got["readdy/observables/n_particles/data"], counts)
    np.testing.assert_array_equal(got["readdy/observables/n_particles/time"], steps)
    rec, lim = got["readdy/trajectory/records"], got["readdy/trajectory/limits"]
    assert rec.dtype.names == ("id", "typeId", "flavor", "pos") and rec.dtype["typeId"] == np.uint16
    np.testing.assert_array_equal(lim, [[0, 4], [4, 10], [10, 15]])
    for k, (pos, types, ids) in enumerate(frames):
        a, b = lim[k]
        np.testing.assert_array_equal(rec["pos"][a:b], pos)
        np.testing.assert_array_equal(rec["id"][a:b], ids)
        np.testing.assert_array_equal(rec["typeId"][a:b], types)


def test_batch_layout_has_one_series_per_replica():
    counts = np.arange(2 * 3 * 2).reshape(2, 3, 2)
    lay = io.batch_n_particles_layout([0, 10], counts)
    for r in range(3):
        np.testing.assert_array_equal(lay[f"readdy/observables/n_particles/replica_{r}/data"], counts[:, r, :])
