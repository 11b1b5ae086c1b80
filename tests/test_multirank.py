"""Sample-range decomposition over ranks (src/mpi.jl:49-54, 104-127) with a real
torch.distributed all-reduce (gloo, world size 2, CPU).  The per-rank integrals come from the
CPU oracle through a stand-in for the device, so the host-side rank logic of qiw.inchworm --
rank_sub_range, Sobol index offsets, rank weights and the packed all-reduce -- is what is
under test."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp


class OracleDevice:
    """Duck-typed stand-in for qiw.device.Device backed by the CPU oracle."""

    def __init__(self):
        self.groups = {}
        self.group_info = {}

    def set_problem(self, exp):
        import oracle as orc
        self.pb = orc.OracleProblem(exp)
        self.exp = exp
        self.groups.clear()
        return None

    def set_ppgf(self, P):
        for s, P_s in enumerate(P):
            self.pb.P_data[s] = np.ascontiguousarray(P_s.data.copy())

    def sobol(self, D):
        from qiw.sobol import direction_numbers
        return direction_numbers(D)

    def create_group(self, kind, order, n_pts_after, tops, corr=None):
        gid = len(self.groups)
        okind = {0: "bold", 1: "bare", 2: "corr", 3: "sigma"}[kind]
        self.groups[gid] = (okind, order, n_pts_after, [(t.pairs, t.parity) for t in tops], corr)
        self.group_info[gid] = (kind, order, n_pts_after)
        return gid

    def integrate(self, works, precision=0):
        out = []
        for w in works:
            okind, order, npa, tops, corr = self.groups[w.group]
            out.append(self.pb.integrate(okind, order, npa, tops, w.t_i, w.t_w, w.t_f, w.n_total, corr=corr,
                                         m=w.sobol_m, x0=w.sobol_x0, sample_range=(w.first_index, w.n_samples)))
        return out


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "qinchworm.jl_gb300"), os.path.join(root, "oracle"), os.path.join(root, "tests")):
        sys.path.insert(0, p)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from qiw import models
    from qiw.inchworm import inchworm, TorchComm
    from test_multirank import OracleDevice
    exp = models.anderson(n_tau=8)
    inchworm(exp, range(0, 3), range(0, 3), 32, dev=OracleDevice(), comm=TorchComm())
    q.put((rank, [P_s.data.copy() for P_s in exp.P]))
    dist.destroy_process_group()


def _worker_corr_diff(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "qinchworm.jl_gb300"), os.path.join(root, "oracle"), os.path.join(root, "tests")):
        sys.path.insert(0, p)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from qiw import models
    from qiw.inchworm import correlator_2p, diff_inchworm, TorchComm
    from test_multirank import OracleDevice
    exp = models.anderson(n_tau=8, corr=True)
    G = correlator_2p(exp, range(0, 3), 32, dev=OracleDevice(), comm=TorchComm())
    exp_d = models.anderson(n_tau=8)
    diff_inchworm(exp_d, range(0, 3), 32, dev=OracleDevice(), comm=TorchComm())
    q.put((rank, ([np.asarray(g) for g in G], [P_s.data.copy() for P_s in exp_d.P])))
    dist.destroy_process_group()


def _randomized_step(comm=None):
    """One inch step with scrambled sequences and an early stop, through OracleDevice."""
    from qiw import models, sobol
    from qiw.diagrammatics import get_topologies_at_order
    from qiw.inchworm import Comm, RandomizationParams, TopologiesInputData, inchworm_step
    exp = models.anderson(n_tau=8)
    g = exp.grid
    rp = RandomizationParams(rng=sobol.NumpyBitRNG(5), N_seqs=5, target_std=3e-3)
    tds = [TopologiesInputData(o, npa, get_topologies_at_order(o, npa), 32, rp)
           for o in (1, 2) for npa in range(1, 2 * o)]
    _, contribs, stds = inchworm_step(exp, g.tau(0), g.tau(3), g.tau(4), tds, dev=OracleDevice(),
                                      comm=comm or Comm())
    vec = lambda d: np.concatenate([d[o][s][1].ravel() for o in sorted(d) for s in sorted(d[o])])
    return vec(contribs), vec(stds), int(rp.rng.g.integers(1 << 62))


def _worker_randomized(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "qinchworm.jl_gb300"), os.path.join(root, "oracle"), os.path.join(root, "tests")):
        sys.path.insert(0, p)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from qiw.inchworm import TorchComm
    from test_multirank import _randomized_step
    q.put((rank, _randomized_step(TorchComm())))
    dist.destroy_process_group()


def test_two_rank_randomized_step_equals_single_rank():
    """Scrambled sequences with an early stop on target_std: the stop is decided on the
    all-reduced values (src/randomization.jl:95-96 after src/inchworm.jl:190), so both ranks use
    the same sequences as one rank and leave the generator in the same state."""
    res = _run_ranks(_worker_randomized)
    mean, std, nxt = _randomized_step()
    for r in (0, 1):
        m, sd, n = res[r]
        assert np.abs(m - mean).max() <= 1e-13 * np.abs(mean).max()
        assert np.abs(sd - std).max() <= 1e-10 * np.abs(std).max()
        assert n == nxt


def _run_ranks(target, world=2):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    import queue
    import time
    res = {}
    deadline = time.time() + 900
    while len(res) < len(procs) and time.time() < deadline:
        try:
            r, v = q.get(timeout=5)
            res[r] = v
        except queue.Empty:
            if any(p.exitcode not in (None, 0) for p in procs):
                break
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    assert sorted(res) == list(range(world))
    return res


def test_two_rank_correlator_and_diff_inchworm_equal_single_rank():
    """correlator_2p (src/inchworm.jl:868-889) and diff_inchworm! (:573-594) split their samples
    over ranks the same way; two gloo ranks reproduce the single-rank oracle."""
    import oracle as orc
    from qiw import models
    res = _run_ranks(_worker_corr_diff)
    exp = models.anderson(n_tau=8, corr=True)
    want_G = orc.correlator_2p(orc.OracleProblem(exp), range(0, 3), 32)
    pb, _ = orc.diff_inchworm(models.anderson(n_tau=8), range(0, 3), 32)
    for r in (0, 1):
        G, P = res[r]
        for a, b in zip(G, want_G):
            assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()
        for s in range(len(pb.P_data)):
            assert np.abs(P[s] - pb.P_data[s]).max() <= 1e-13 * np.abs(pb.P_data[s]).max()


def test_two_rank_inchworm_equals_single_rank():
    import oracle as orc
    from qiw import models
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    import queue
    import time
    res = {}
    deadline = time.time() + 900
    while len(res) < len(procs) and time.time() < deadline:
        try:
            r, P = q.get(timeout=5)
            res[r] = P
        except queue.Empty:
            if any(p.exitcode not in (None, 0) for p in procs):
                break
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    assert sorted(res) == [0, 1]
    exp = models.anderson(n_tau=8)
    pb = orc.inchworm(exp, range(0, 3), range(0, 3), 32)   # one rank, 32 samples (ranks: 16 + 16)
    for s in range(len(pb.P_data)):
        want = pb.P_data[s]
        for r in (0, 1):
            got = res[r][s]
            assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()


def _bench_steps(comm=None, n_steps=3):
    """bench.py's bare step and regular steps (bench.bare_step / bench.make_step) on a small
    Anderson model through OracleDevice; returns the P tables afterwards."""
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    import bench
    from qiw import models, _lib
    from qiw.inchworm import Comm, _Session
    exp = models.anderson(n_tau=8)
    comm = comm or Comm()
    tds = bench.bold_groups(range(0, 3), 32)   # N_samples * world: each of two ranks takes 16
    ses = _Session(OracleDevice(), exp)
    bench.bare_step(ses, exp, 2, 32, _lib.QIW_PREC_FP64, comm)
    step = bench.make_step(ses, exp, tds, _lib.QIW_PREC_FP64, comm)
    for n in range(1, 1 + n_steps):
        step(n)
    return [P_s.data.copy() for P_s in exp.P]


def _worker_bench(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "qinchworm.jl_gb300"), os.path.join(root, "oracle"), os.path.join(root, "tests")):
        sys.path.insert(0, p)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from qiw.inchworm import TorchComm
    from test_multirank import _bench_steps
    q.put((rank, _bench_steps(TorchComm())))
    dist.destroy_process_group()


def test_two_rank_bench_steps_equal_single_rank():
    """bench.py's torchrun path (weak scaling: each rank a sample range of every group, one
    all-reduce per launch) gives the single-rank P on two gloo ranks."""
    res = _run_ranks(_worker_bench)
    want = _bench_steps()
    for r in (0, 1):
        for a, b in zip(res[r], want):
            assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()


def _worker_shard(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "qinchworm.jl_gb300"), root):
        sys.path.insert(0, p)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from qiw.batch import shard_solves, solve_cost
    specs = bench.batch_solves(2024, 64)
    costs = [solve_cost(p["n_tau"], p["kmax"], p["N"]) for p in specs]
    mine = shard_solves(costs, rank, world)
    shares = [None] * world
    dist.all_gather_object(shares, mine)
    q.put((rank, (shares, costs)))
    dist.destroy_process_group()


def test_batch_solves_shard_over_ranks_without_exchange():
    """The 64 seed-drawn solves of the batch benchmark dealt out whole over gloo ranks: every
    rank computes the same partition on its own (no exchange), the shares are disjoint, cover
    every solve, and no rank carries more than the even share plus the largest single solve."""
    for world in (2, 3):
        res = _run_ranks(_worker_shard, world)
        shares, costs = res[0]
        for r in range(1, world):
            assert res[r][0] == shares
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in s) for s in shares]
        assert max(loads) <= sum(costs) / world + max(costs)
