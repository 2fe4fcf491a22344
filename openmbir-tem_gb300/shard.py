"""y-slab sharding of one HAADF reconstruction over ranks (one GPU per rank).

Voxel slice y touches only its own detector rows, so contiguous slabs of slices own disjoint
blocks of the error sinogram and the ICD sweep needs no sinogram exchange.  The prior couples
neighbouring slices: after each colour phase (red/black in y) every rank publishes its two
boundary planes and takes its neighbours' planes as read-only halos.  The per-view sums of the
gain/offset estimate (jointEstimation, HAADF_ReconstructionEngine_Extra.cpp:419-636) and of the
variance estimate (updateWeights, :795-881) are summed over ranks, solved on the host and
applied by every rank.  This is the reference's y-range task split of updateVoxels
(HAADF_ReconstructionEngine_UpdateVoxels.cpp:666-723) across devices instead of threads, with
the same result as one engine running the whole volume (the colour order makes the slabs
independent within a phase).

Communication goes through torch.distributed on host tensors (gloo): planes and sums are small
(one N_z x N_x plane per neighbour, 6 N_theta doubles) and are exchanged between kernel launches,
so no kernel ever waits on another rank.

Bright field (`run_sharded_bf`) shards the same way one NHICD call at a time, as the reference
splits a call's y range over worker tasks and adds their magnitude maps afterwards
(BFReconstructionEngine_Extra.cpp:624-752): each call's per-line update magnitudes are added
over ranks, so every rank derives the same non-homogeneous lists; the offset and variance sums
and the stop rule's volume sum are added over ranks too.

Backends: `EngineBackend` (the engine's C ABI, one GPU per rank; the engine holds the whole
problem), `OwnedSlabBackend` (the engine holds only the rank's slab, one halo plane on each side
and their detector rows: the device memory of one slab) and, for tests on CPU ranks, any object
with the same methods (tests use the FP64 oracle).
"""
import numpy as np


def slabs(n_y, world):
    """Contiguous slabs [y0, y1) per rank; sizes differ by at most one slice."""
    counts = [n_y // world + (1 if r < n_y % world else 0) for r in range(world)]
    out, y = [], 0
    for c in counts:
        out.append((y, y + c))
        y += c
    return out


def check_slab_rows(rows, bounds):
    """Slabs own their detector rows only when no two neighbouring slabs' edge slices share a
    row.  rows[y] = (first detector row, row count) of slice y's voxel-line response
    (storeVoxelResponse, HAADF_ReconstructionEngine_Extra.cpp:329-404); at delta_xy = delta_t
    each slice has exactly its own row, but other pixel shapes let slices y and y+1 share one.
    Raises ValueError naming the first shared boundary (every rank sees the same rows and
    bounds, so every rank raises before any exchange)."""
    for (a0, a1), (b0, b1) in zip(bounds[:-1], bounds[1:]):
        if a1 <= a0 or b1 <= b0:
            continue
        last, first = rows[a1 - 1], rows[b0]
        if last[1] > 0 and first[1] > 0 and last[0] + last[1] > first[0]:
            raise ValueError(f"slabs [{a0}, {a1}) and [{b0}, {b1}) share detector rows "
                             f"(slice {a1 - 1} ends at row {last[0] + last[1] - 1}, slice {b0} "
                             f"starts at row {first[0]})")


def solve_gain_offset(sums, target_gain):
    """The Lagrange solve of jointEstimation (HAADF_ReconstructionEngine_Extra.cpp:521-598) from
    the six per-view sums [theta][6] = (y w, w, yh w, yh w y, y^2 w, yh^2 w); mean gain fixed to
    target_gain.  Same operations in the same order as the engine's host solve."""
    s = np.asarray(sums, np.float64).reshape(-1, 6)
    nt = s.shape[0]
    q0, q1, b0 = s[:, 5], s[:, 2], s[:, 3]
    d1 = [s[v, 0] / s[v, 1] for v in range(nt)]
    d2 = [s[v, 2] / s[v, 1] for v in range(nt)]
    sum1 = 0.0
    sum2 = 0.0
    for v in range(nt):
        sum1 += (1.0 / (q0[v] - q1[v] * d2[v]))
        sum2 += ((b0[v] - q1[v] * d1[v]) / (q0[v] - q1[v] * d2[v]))
    lm = (-nt * target_gain + sum2) / sum1
    gain = np.empty(nt)
    offset = np.empty(nt)
    for v in range(nt):
        gain[v] = (-1 * lm - q1[v] * d1[v] + b0[v]) / (q0[v] - q1[v] * d2[v])
        offset[v] = d1[v] - d2[v] * gain[v]
    return gain, offset


class EngineBackend:
    """One rank's engine (C ABI).  The engine holds the whole problem; only its slab is swept
    and summed."""

    def __init__(self, engine):
        self.e = engine

    def dims(self):
        return self.e.dims()

    def set_slab(self, y0, y1):
        self.e.set_slab(y0, y1)

    def sweep_colour(self, colour, outer, inner):
        return self.e.sweep_colour(colour, outer, inner)

    def get_planes(self, y, n):
        return self.e.get_planes(y, n)

    def set_planes(self, y, planes):
        self.e.set_planes(y, planes)

    def view_sums(self, kind):
        return self.e.view_sums(kind)

    def apply_nuisance(self, gain=None, offset=None, variance=None):
        self.e.apply_nuisance(gain, offset, variance)

    def bf_call_begin(self, outer, inner):
        self.e.bf_call_begin(outer, inner)

    def bf_call_magnitudes(self):
        return self.e.bf_call_magnitudes()

    def bf_call_end(self, magnitudes):
        self.e.bf_call_end(magnitudes)

    def bf_slab_sums(self, kind):
        return self.e.bf_slab_sums(kind)

    def bf_slab_apply(self, kind, sums):
        self.e.bf_slab_apply(kind, sums)

    def roi_sums(self):
        return self.e.roi_sums()


def owned_slab(n_y, world, rank):
    """This rank's slab [y0, y1) and the slices [base, top) its engine holds: the slab plus one
    halo plane on each side, the lower end rounded down to an even slice so that the engine's
    local slice parity is the global one (the red/black colours keep their meaning)."""
    y0, y1 = slabs(n_y, world)[rank]
    base = max(0, y0 - 1)
    base -= base & 1
    return (y0, y1), base, min(n_y, y1 + 1)


class OwnedSlabBackend:
    """A rank's engine built on its own slices only (`owned_slab`): the tilt series' detector
    rows of slices [base, top) as its sinogram, the initial nuisance estimated from the whole
    series (so that every rank starts where one engine would), and the drivers' global slice
    indices mapped to the engine's.  Make it with `make`."""

    def __init__(self, engine, dims, base):
        self.e = engine
        self.dims_g = tuple(dims)
        self.base = base

    @classmethod
    def make(cls, mbir, params, counts, tilts, world, rank, rows_per_slice=1, delta_r=1.0,
             delta_t=1.0):
        """counts [theta][r][t] of the whole series; rows_per_slice = delta_xy / delta_t."""
        import numpy as _np
        with mbir.Engine(params) as full:  # host only: geometry and the initial nuisance
            full.set_sinogram(counts, tilts, delta_r, delta_t)
            dims = full.dims()
            gain, offset, var = full.nuisance()
        (y0, y1), base, top = owned_slab(dims[2], world, rank)
        f = rows_per_slice
        sub = _np.ascontiguousarray(counts[:, :, f * base:f * top])
        e = mbir.Engine(params)
        e.set_sinogram(sub, tilts, delta_r, delta_t)
        e.set_initial_nuisance(gain, offset, var)
        e.prepare()
        return cls(e, dims, base)

    def close(self):
        self.e.close()

    def dims(self):
        return self.dims_g

    def set_slab(self, y0, y1):
        self.e.set_slab(y0 - self.base, y1 - self.base)

    def sweep_colour(self, colour, outer, inner):
        return self.e.sweep_colour(colour, outer, inner)

    def get_planes(self, y, n):
        return self.e.get_planes(y - self.base, n)

    def set_planes(self, y, planes):
        self.e.set_planes(y - self.base, planes)

    def view_sums(self, kind):
        return self.e.view_sums(kind)

    def apply_nuisance(self, gain=None, offset=None, variance=None):
        self.e.apply_nuisance(gain, offset, variance)

    def bf_call_begin(self, outer, inner):
        self.e.bf_call_begin(outer, inner)

    def bf_call_magnitudes(self):
        return self.e.bf_call_magnitudes()

    def bf_call_end(self, magnitudes):
        self.e.bf_call_end(magnitudes)

    def bf_slab_sums(self, kind):
        return self.e.bf_slab_sums(kind)

    def bf_slab_apply(self, kind, sums):
        self.e.bf_slab_apply(kind, sums)

    def roi_sums(self):
        return self.e.roi_sums()


def _exchange(dist, backend, y0, y1, n_y, nz, nx):
    """Every rank publishes its first and last plane; ranks take their neighbours' planes."""
    import torch
    world = dist.get_world_size()
    rank = dist.get_rank()
    dtype = getattr(backend, "plane_dtype", np.float32)
    mine = np.zeros((2, nz, nx), dtype)
    if y1 > y0:
        mine[0] = backend.get_planes(y0, 1)[0]
        mine[1] = backend.get_planes(y1 - 1, 1)[0]
    out = [torch.zeros((2, nz, nx), dtype=torch.from_numpy(mine).dtype) for _ in range(world)]
    dist.all_gather(out, torch.from_numpy(mine))
    bounds = slabs(n_y, world)
    if rank > 0 and y0 > 0:
        left = out[rank - 1].numpy()
        if bounds[rank - 1][1] == y0:
            backend.set_planes(y0 - 1, left[1:2])
    if rank + 1 < world and y1 < n_y:
        right = out[rank + 1].numpy()
        if bounds[rank + 1][0] == y1:
            backend.set_planes(y1, right[0:1])


def _allreduce(dist, arr):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(arr, np.float64))
    dist.all_reduce(t)
    return t.numpy().copy()


def run_sharded(dist, backend, n_outer, target_gain=1.0, joint_estimation=True,
                noise_model=True):
    """Outer iterations of the parallel-order reconstruction on this rank's slab: per outer
    iteration one sweep (colour 0, halo exchange, colour 1, halo exchange), then the gain/offset
    and variance updates from sums over all ranks.  Returns the rank's (y0, y1) and the summed
    sweep statistics (sum |dx|, sum |x| over the ROI, zero-skipped, updated) per sweep."""
    nz, nx, n_y, n_theta, n_r, n_t = backend.dims()
    world = dist.get_world_size()
    rank = dist.get_rank()
    bounds = slabs(n_y, world)
    if hasattr(backend, "slice_rows"):
        check_slab_rows(backend.slice_rows(), bounds)
    y0, y1 = bounds[rank]
    backend.set_slab(y0, y1)
    history = []
    for outer in range(n_outer):
        st = np.zeros(4)
        for colour in (0, 1):
            st += backend.sweep_colour(colour, outer, 0)
            _exchange(dist, backend, y0, y1, n_y, nz, nx)
        history.append(_allreduce(dist, st))
        if joint_estimation:
            gain, offset = solve_gain_offset(_allreduce(dist, backend.view_sums(0)), target_gain)
            backend.apply_nuisance(gain, offset, None)
        if noise_model:
            var = _allreduce(dist, backend.view_sums(1)) / (n_r * n_t)
            backend.apply_nuisance(None, None, var)
    return (y0, y1), history


def _allreduce_int(dist, arr):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(arr).astype(np.int64))
    dist.all_reduce(t)
    return t.numpy().astype(np.uint64)


# NHICD list counts (MBIR::Constants k_NumHomogeniousIter / k_NumNonHomogeniousIter)
NUM_NON_HOMOGENEOUS = 20


def run_sharded_bf(dist, backend, n_outer, stop_threshold=0.0, reduction_factor=1.0,
                   joint_estimation=True, noise_estimation=True, nhicd=True):
    """A bright-field reconstruction on this rank's slab with one NHICD call per outer
    iteration (BFReconstructionEngine::execute with one inner iteration, so the Bragg threshold
    keeps its requested value, BFReconstructionEngine.cpp:595-858): per call both colours with
    the halo exchange after each, the call's magnitudes added over ranks, the stop rule on the
    ROI sums (stopCriteria, _Extra.cpp:1217-1273), then the offset and variance updates from
    sums over all ranks.  Returns the rank's (y0, y1) and the summed statistics per call."""
    nz, nx, n_y = backend.dims()[:3]
    world = dist.get_world_size()
    rank = dist.get_rank()
    bounds = slabs(n_y, world)
    if hasattr(backend, "slice_rows"):
        check_slab_rows(backend.slice_rows(), bounds)
    y0, y1 = bounds[rank]
    backend.set_slab(y0, y1)
    history = []
    prev_mag, stop, calls = 0.0, stop_threshold, 0
    for outer in range(n_outer):
        eff = calls
        backend.bf_call_begin(outer, 0)
        st = np.zeros(4)
        for colour in (0, 1):
            st += backend.sweep_colour(colour, outer, 0)
            _exchange(dist, backend, y0, y1, n_y, nz, nx)
        backend.bf_call_end(_allreduce_int(dist, backend.bf_call_magnitudes()))
        calls += 1
        history.append(_allreduce(dist, st))
        roi = backend.roi_sums()
        status = 1
        check = (eff % NUM_NON_HOMOGENEOUS == 0) if nhicd else True
        if check and eff > 0 and prev_mag > 0 and abs(roi[0]) / abs(prev_mag) < stop:
            stop *= reduction_factor
            status = 0
        if not nhicd or eff % NUM_NON_HOMOGENEOUS == 0:
            prev_mag = float(_allreduce(dist, roi[1:2])[0])
        if status == 0 and outer >= 1:
            break
        if n_outer > 1:
            if joint_estimation:
                backend.bf_slab_apply(2, _allreduce(dist, backend.bf_slab_sums(2)))
            if noise_estimation:
                backend.bf_slab_apply(3, _allreduce(dist, backend.bf_slab_sums(3)))
    return (y0, y1), history


def gather_volume(dist, backend, y0, y1):
    """The full volume [z][x][y] on every rank, assembled from the ranks' slabs."""
    import torch
    nz, nx, n_y = backend.dims()[:3]
    mine = np.zeros((n_y, nz, nx), np.float32)
    if y1 > y0:
        mine[y0:y1] = backend.get_planes(y0, y1 - y0)
    t = torch.from_numpy(mine)
    dist.all_reduce(t)
    return t.numpy().transpose(1, 2, 0).copy()
