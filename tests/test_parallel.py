"""Shot sharding and the distributed FWI driver (fwi_cuda_gb300/parallel.py)
with two gloo ranks on CPU.  The plan behind the driver is a stand-in that
computes with the FP64 oracle, so the test checks the driver's reduction and
line-search logic against the single-process oracle FWI."""
import os
import socket
import tempfile

import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import parallel


def test_shard_shots_partition():
    for nshot in (1, 5, 8, 64):
        for world in (1, 2, 3, 8):
            parts = [parallel.shard_shots(nshot, world, r) for r in range(world)]
            flat = [s for p in parts for s in p]
            assert flat == list(range(nshot))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1


def test_shard_survey_remaps_sources():
    sv, _, _ = helpers.case(nshot=5)
    loc = parallel.shard_survey(sv, [2, 3])
    assert loc.nshot == 2
    assert list(loc.src_shot_to_fire) == [0, 1]
    assert list(loc.x_src) == list(np.asarray(sv.x_src)[[2, 3]])


class OraclePlan:
    """The engine Plan's FWI-piece interface, computed by the FP64 oracle."""

    def __init__(self, orc, sv, model, uz, ux):
        self.orc, self.sv, self.uz, self.ux = orc, sv, uz, ux
        self.m = [np.array(a, np.float64) for a in model]
        self.g = [np.zeros((sv.nz, sv.nx)) for _ in range(3)]

    def reset_gradient(self):
        self.g = [np.zeros_like(x) for x in self.g]

    def gradient(self):
        L2, c, _ = helpers.oracle_gradient(self.orc, self.sv, self.m, self.uz, self.ux)
        self.g = [a + b for a, b in zip(self.g, c)]
        return L2, [x.copy() for x in self.g]

    def set_gradient(self, *g):
        self.g = [np.array(x) for x in g]

    def get_gradient(self):
        return [x.copy() for x in self.g]

    def save_model(self):
        self.saved = [x.copy() for x in self.m]

    def taper_gradient(self):
        sv = self.sv
        snap = (sv.snap_z1, sv.snap_z2, sv.snap_x1, sv.snap_x2)
        self.g = [self.orc.taper2(x, snap, sv.taper) for x in self.g]

    def _updated(self, step, rho_min):
        o, (l0, m0, r0) = self.orc, self.saved
        return [o.update_mat2(l0, self.g[0], 4.8e10, 0.0, step),
                o.update_mat2(m0, self.g[1], 2.7e10, 0.0, step),
                o.update_mat2(r0, self.g[2], 3000.0, rho_min, 0.5 * step)]

    def trial_misfit(self, step):
        m = self._updated(step, 1.5)
        uz, ux = self.orc.simulate_fwd(self.sv, *m)
        return sum(self.orc.adjsrc2(uz[s], ux[s], self.uz[s], self.ux[s], self.sv.dt)[0]
                   for s in range(self.sv.nshot))

    def update_model(self, step):
        self.m = self._updated(step, 1.25)


def _worker(rank, world, port, out):
    import torch.distributed as dist
    from oracle import oracle as O
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    orc = O.oracle()
    orc.set_threads(1)
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=3, nt=220, nz=51, nx=71,
                                  npml=8, nrec=12, imaging_sign=1)
    uz, ux = orc.simulate_fwd(sv, *true)
    shots = parallel.shard_shots(sv.nshot, world, rank)
    loc = parallel.shard_survey(sv, shots)
    drv = parallel.DistributedFWI(OraclePlan(orc, loc, init, uz[shots], ux[shots]), sv.nz, sv.nx,
                                  parallel.torch_allreduce())
    step, rows = 0.01, []
    for _ in range(2):
        r = drv.iteration(step)
        step = r["step"]
        rows.append([r["L2"], r["step"], r["ntrials"]])
    if rank == 0:
        np.save(out, np.array(rows))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_fwi_matches_single_process_oracle(orc):
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = os.path.join(tempfile.mkdtemp(), "rows.npy")
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    rows = np.load(out)
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=3, nt=220, nz=51, nx=71,
                                  npml=8, nrec=12, imaging_sign=1)
    uz, ux = orc.simulate_fwd(sv, *true)
    r = orc.simulate_fwi(sv, *init, uz, ux, niter=2)
    assert r["rc"] == 0
    np.testing.assert_allclose(rows[:, 0], r["L2"], rtol=1e-11)
    np.testing.assert_allclose(rows[:, 1], r["step"], rtol=1e-9)
    assert list(rows[:, 2].astype(int)) == list(r["trials"])


def _silent_worker(rank, world, port, out):
    # shot 1 (rank 1's) has no source: the summed gradient is NaN, so is
    # every rank's first trial misfit after the all-reduce, and every rank
    # leaves the step search at that same trial (none is left waiting in a
    # collective)
    import datetime
    import torch.distributed as dist
    from fwi_cuda_gb300 import _lib
    from oracle import oracle as O
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world, timeout=datetime.timedelta(seconds=60))
    orc = O.oracle()
    orc.set_threads(1)
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=2, nt=120, nz=41, nx=61,
                                  npml=8, nrec=6, imaging_sign=1)
    sv.src_shot_to_fire = np.zeros(sv.nsrc, np.int32)
    sv.finalize()
    uz, ux = orc.simulate_fwd(sv, *true)
    shots = parallel.shard_shots(sv.nshot, world, rank)
    loc = parallel.shard_survey(sv, shots)
    drv = parallel.DistributedFWI(OraclePlan(orc, loc, init, uz[shots], ux[shots]), sv.nz, sv.nx,
                                  parallel.torch_allreduce())
    try:
        drv.iteration(0.01)
        status = 0
    except _lib.PSVError as e:
        status = e.status
    got = parallel.torch_allreduce()(np.array([float(status), 1.0]))
    if rank == 0:
        np.save(out, np.array([status, got[0], got[1]]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_fwi_stops_together_on_a_nan_misfit():
    import torch.multiprocessing as mp
    from fwi_cuda_gb300 import _lib
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = os.path.join(tempfile.mkdtemp(), "status.npy")
    mp.spawn(_silent_worker, args=(2, port, out), nprocs=2, join=True)
    status, total, ranks = np.load(out)
    assert status == _lib.PSV_ERR_STEP_SEARCH and ranks == 2
    assert total == 2 * _lib.PSV_ERR_STEP_SEARCH  # the same failure on both ranks


class FailingPlan(OraclePlan):
    """OraclePlan whose gradient or first trial forward fails on one rank."""

    def __init__(self, *a, fail_in=None, status=None):
        super().__init__(*a)
        self.fail_in, self.status = fail_in, status

    def gradient(self):
        from fwi_cuda_gb300 import _lib
        if self.fail_in == "gradient":
            raise _lib.PSVError(self.status, "planted gradient failure")
        return super().gradient()

    def trial_misfit(self, step):
        from fwi_cuda_gb300 import _lib
        if self.fail_in == "trial":
            raise _lib.PSVError(self.status, "planted trial failure")
        return super().trial_misfit(step)


def _one_rank_fails_worker(rank, world, port, out, where):
    # only rank 1 fails (its gradient, or its first trial forward); rank 0
    # must leave the iteration with the same status instead of waiting in
    # the next all-reduce (the 60 s process-group timeout would end it with
    # a different error)
    import datetime
    import torch.distributed as dist
    from fwi_cuda_gb300 import _lib
    from oracle import oracle as O
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world, timeout=datetime.timedelta(seconds=60))
    orc = O.oracle()
    orc.set_threads(1)
    sv, true, init = helpers.case(fdorder=4, stencil="holberg", nshot=2, nt=120, nz=41, nx=61,
                                  npml=8, nrec=6, imaging_sign=1)
    uz, ux = orc.simulate_fwd(sv, *true)
    shots = parallel.shard_shots(sv.nshot, world, rank)
    loc = parallel.shard_survey(sv, shots)
    plan = FailingPlan(orc, loc, init, uz[shots], ux[shots],
                       fail_in=where if rank == 1 else None, status=_lib.PSV_ERR_OOM)
    drv = parallel.DistributedFWI(plan, sv.nz, sv.nx, parallel.torch_allreduce())
    try:
        drv.iteration(0.01)
        status = 0
    except _lib.PSVError as e:
        status = e.status
    got = parallel.torch_allreduce()(np.array([float(status), 1.0]))
    if rank == 0:
        np.save(out, np.array([status, got[0], got[1]]))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("where", ["gradient", "trial"])
def test_two_rank_fwi_leaves_together_when_one_rank_fails(where):
    import torch.multiprocessing as mp
    from fwi_cuda_gb300 import _lib
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = os.path.join(tempfile.mkdtemp(), "status.npy")
    mp.spawn(_one_rank_fails_worker, args=(2, port, out, where), nprocs=2, join=True)
    status, total, ranks = np.load(out)
    assert ranks == 2
    assert status == _lib.PSV_ERR_OOM                 # rank 0 did not fail itself
    assert total == 2 * _lib.PSV_ERR_OOM              # both ranks report the failure
