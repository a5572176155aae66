"""Observable output in ReaDDy's file layout, without HDF5.

ReaDDy writes observables into an HDF5 file: a time series per observable under /readdy/observables/<name>
with a "data" dataset and a "time" dataset appended together (TimeSeriesWriter,
include/readdy/model/observables/io/TimeSeriesWriter.h:56-92; NParticles.cpp:75-90), and trajectories under
/readdy/trajectory as flat "records" of (id, typeId, flavor, pos) entries with per-frame [begin, end)
"limits" and "time" (FlatTrajectory, readdy/main/model/observables/Trajectory.cpp:100-160; entry layout
observables/Types.cpp:79-88).  The HDF5 library is not available here, so these functions build the same
datasets -- same paths, same element types and shapes -- as numpy arrays, and save_layout writes them to
a .npz archive whose keys are the dataset paths.  A tool that reads ReaDDy's files can read the arrays by
the same names.
"""
from __future__ import annotations

import numpy as np

OBSERVABLES_GROUP_PATH = "readdy/observables"
TRAJECTORY_GROUP_PATH = "readdy/trajectory"

# TrajectoryEntry (include/readdy/model/observables/io/TrajectoryEntry.h:55-65): ParticleId is unsigned
# long, ParticleTypeId unsigned short, ParticleFlavor uint8, positions in the reference's double scalar
TRAJECTORY_ENTRY = np.dtype([("id", np.uint64), ("typeId", np.uint16), ("flavor", np.uint8), ("pos", np.float64, (3,))])


def n_particles_layout(steps, counts, name: str = "n_particles") -> dict:
    """NParticles time series: data (n_records, n_types) of std::size_t, time (n_records,) of TimeStep."""
    counts = np.asarray(counts)
    group = f"{OBSERVABLES_GROUP_PATH}/{name}"
    return {f"{group}/data": counts.astype(np.uint64), f"{group}/time": np.asarray(steps, np.uint64)}


def batch_n_particles_layout(steps, counts, name: str = "n_particles") -> dict:
    """One NParticles time series per replica of a batch (counts of shape (n_records, n_replicas, n_types)),
    under <name>/replica_<r>."""
    counts = np.asarray(counts)
    out = {}
    for r in range(counts.shape[1]):
        out.update(n_particles_layout(steps, counts[:, r, :], f"{name}/replica_{r}"))
    return out


def flat_trajectory_layout(frames, steps, name: str = "") -> dict:
    """FlatTrajectory: `frames` is a list of (positions (n, 3), types (n,), ids (n,)) snapshots taken at
    `steps`.  records holds every frame's entries one after another, limits[k] = [begin, end) of frame k."""
    group = TRAJECTORY_GROUP_PATH + (f"/{name}" if name else "")
    sizes = [len(f[0]) for f in frames]
    records = np.zeros(sum(sizes), TRAJECTORY_ENTRY)
    limits = np.zeros((len(frames), 2), np.uint64)
    at = 0
    for k, (pos, types, ids) in enumerate(frames):
        n = len(pos)
        records["id"][at:at + n] = np.asarray(ids, np.uint64)
        records["typeId"][at:at + n] = np.asarray(types, np.uint16)
        records["pos"][at:at + n] = np.asarray(pos, np.float64)
        limits[k] = (at, at + n)
        at += n
    return {f"{group}/records": records, f"{group}/limits": limits, f"{group}/time": np.asarray(steps, np.uint64)}


def batch_trajectory_layout(steps, frames, replicas, name: str = "") -> dict:
    """One FlatTrajectory per recorded replica of a batch, under <name>/replica_<r>: `frames[f][k]` is the
    (positions, types, ids) snapshot of replica replicas[k] at steps[f] (ReplicaBatch.poll_trajectory)."""
    out = {}
    for k, r in enumerate(replicas):
        sub = f"{name}/replica_{int(r)}" if name else f"replica_{int(r)}"
        out.update(flat_trajectory_layout([fr[k] for fr in frames], steps, sub))
    return out


def save_layout(path: str, *layouts: dict) -> None:
    """Writes the datasets of the given layouts into one .npz archive keyed by dataset path."""
    merged = {}
    for layout in layouts:
        merged.update(layout)
    np.savez(path, **merged)


def load_layout(path: str) -> dict:
    with np.load(path, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}
