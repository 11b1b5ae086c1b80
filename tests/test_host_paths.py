"""Host-side result handling of qiw.device.Device, without a GPU: the C library is replaced by a
stand-in that writes a deterministic result buffer, so the unpacking, the packed layout and
the correlator's trace extraction are checked against each other; and the call sequence and
keep/drop decisions of fitting several groups' warps together, on a stand-in device."""
import ctypes as C

import numpy as np

from qiw import _lib, models
from qiw.device import Device, Work


class _FakeLib:
    """qiw_integrate writes value k * 1e-3 + i * (k % 7) into double k of the output."""

    def qiw_integrate(self, h, n, descs, precision, out):
        rs = self.rs
        buf = (C.c_double * (2 * rs * n)).from_address(out)
        for k in range(2 * rs * n):
            buf[k] = k * 1e-3 if k % 2 == 0 else float((k // 2) % 7)
        return _lib.QIW_OK

    def qiw_integrate_sample_norms(self, h, n, descs, precision, out, norms):
        self.qiw_integrate(h, n, descs, precision, out)
        total = sum(descs[i].n_samples for i in range(n))
        buf = (C.c_double * total).from_address(norms)
        for k in range(total):
            buf[k] = float(k)
        return _lib.QIW_OK

    def qiw_integrate_samples_batch(self, h, n, descs, precision, out, samples):
        self.qiw_integrate(h, n, descs, precision, out)
        total = sum(descs[i].n_samples for i in range(n)) * self.rs
        buf = (C.c_double * total).from_address(samples)
        for k in range(total):
            buf[k] = float(k)
        return _lib.QIW_OK

    def qiw_problem_set(self, h, d):
        return _lib.QIW_OK

    def qiw_ppgf_set(self, h, p):
        return _lib.QIW_OK

    def qiw_group_create(self, h, gd, gid):
        gid._obj.value = self.next_gid
        self.next_gid += 1
        return _lib.QIW_OK


def _device(exp):
    dev = Device.__new__(Device)   # no context: only the host-side methods are used
    dev.lib = _FakeLib()
    dev.lib.next_gid = 0
    dev.h = None
    dev.group_info = {}
    dev._sobol_cache = {}
    dev.set_problem(exp)
    dev.lib.rs = int(np.sum(dev.packed.dims ** 2))
    return dev


def test_integrate_packed_has_the_unpacked_layout():
    exp = models.eg_discrete_bath(n_tau=8)   # sector dimensions 1, 2 and 4
    dev = _device(exp)
    works = [Work(0, 0.0, 0.1, 0.2, 0, 8, 8) for _ in range(3)]
    blocks = dev.integrate(works)
    packed = dev.integrate_packed(works)
    for i, bl in enumerate(blocks):
        assert np.array_equal(np.concatenate([b.ravel(order="F") for b in bl]), packed[i])


def test_correlator_traces_from_packed_results_equal_block_traces():
    from qiw.inchworm import correlator_2p
    exp = models.eg_discrete_bath(n_tau=6, corr=True)
    a = correlator_2p(exp, range(0, 2), 8, dev=_device(exp))
    b_dev = _device(exp)

    class NoPacked:   # the same device without integrate_packed: the block path
        def __init__(self, d):
            self._d = d

        def __getattr__(self, name):
            if name == "integrate_packed":
                raise AttributeError(name)
            return getattr(self._d, name)

    b = correlator_2p(exp, range(0, 2), 8, dev=NoPacked(b_dev))
    for x, y in zip(a, b):
        assert np.allclose(x, y, rtol=1e-14, atol=0)


def test_inchworm_steps_from_packed_results_equal_block_path():
    from qiw.inchworm import inchworm

    class NoPacked:
        def __init__(self, d):
            self._d = d

        def __getattr__(self, name):
            if name == "integrate_packed":
                raise AttributeError(name)
            return getattr(self._d, name)

    res = []
    for wrap in (lambda d: d, NoPacked):
        exp = models.eg_discrete_bath(n_tau=5)
        # the stand-in results are not a physical P: keep normalize! away from log(<= 0)
        dev = _device(exp)
        dev.lib.qiw_integrate = _positive_integrate(dev.lib.rs)
        inchworm(exp, range(0, 2), range(0, 2), 8, dev=wrap(dev))
        res.append([P.data.copy() for P in exp.P])
    for x, y in zip(*res):
        assert np.array_equal(x, y)


def _positive_integrate(rs):
    """Results -i * (1e-3 + k 1e-6) on every entry k (P(tau) stays of the form -i * positive)."""
    def f(h, n, descs, precision, out):
        buf = (C.c_double * (2 * rs * n)).from_address(out)
        for k in range(rs * n):
            buf[2 * k] = 0.0
            buf[2 * k + 1] = -(1e-3 + k * 1e-6)
        return _lib.QIW_OK
    return f


class _FitDevice:
    """Stand-in for qiw.device.Device in fit_group_warps: deterministic per-sample norms and
    replica results (the warped replicas of group 3 vary less than its plain ones, those of
    group 2 more), and a record of the calls."""

    def __init__(self):
        self.group_info = {0: (1, 0, 0), 1: (1, 1, 1), 2: (1, 2, 2), 3: (1, 2, 3), 4: (1, 1, 1)}
        self.calls = []
        self.next_wid = 100

    def integrate_sample_norms(self, works, precision):
        self.calls.append(("norms", [w.group for w in works], [w.n_samples for w in works]))
        norms = [np.zeros(w.n_samples) if w.group == 4 else np.linspace(1.0, 2.0, w.n_samples) for w in works]
        return None, norms

    def warp_create(self, D, seed=0, uniform_mix=None):
        self.calls.append(("create", D, seed, uniform_mix))
        self.next_wid += 1
        return self.next_wid

    def warp_train_batch(self, wids, xs, ws, steps, batch, lr):
        self.calls.append(("train", list(wids), [x.shape for x in xs], [len(w) for w in ws], steps, batch))
        return np.arange(len(wids), dtype=float) * 0.1

    def integrate(self, works, precision, warps=None):
        self.calls.append(("integrate", [w.group for w in works], warps is not None))
        out = []
        for k, w in enumerate(works):
            r = k % 4   # replica index within the group (R = 4 below)
            spread = {2: 1.0 if warps is None else 3.0, 3: 1.0 if warps is None else 0.2}.get(w.group, 1.0)
            out.append([np.array([[1.0 + spread * (r - 1.5)]])])
        return out


def test_fit_group_warps_orchestration_without_a_gpu():
    """fit_group_warps: order-0 groups and groups whose samples are all zero get no warp; the
    others share one norms launch, one concurrent training call and one launch per estimator,
    and keep their warp only where the warped replicas vary less (gain above min_gain = 1)."""
    from qiw import warp as qwarp
    dev = _FitDevice()
    works = [Work(g, 0.0, 0.5, 1.0, 0, 0, 0) for g in (0, 1, 2, 3, 4)]
    fits = qwarp.fit_group_warps(dev, works, n_train=256, steps=7, batch=64, R=4, N_test=32)
    assert [f.warp_id is None for f in fits] == [True, True, True, False, True]
    assert fits[0].gain == 1.0 and fits[4].gain == 1.0 and np.isclose(fits[1].gain, 1.0)
    assert np.isclose(fits[2].gain, 1 / 9) and np.isclose(fits[3].gain, 25.0)
    kinds = [c[0] for c in dev.calls]
    assert kinds == ["norms", "create", "create", "create", "train", "integrate", "integrate"]
    assert dev.calls[0][1] == [1, 2, 3, 4] and dev.calls[0][2] == [256] * 4
    train = dev.calls[4]
    assert train[2] == [(256, 2), (256, 4), (256, 4)] and train[3] == [256] * 3 and train[4:] == (7, 64)
    assert dev.calls[5] == ("integrate", [1] * 4 + [2] * 4 + [3] * 4, False)
    assert dev.calls[6] == ("integrate", [1] * 4 + [2] * 4 + [3] * 4, True)
    assert [f.loss for f in fits] == [0.0, 0.0, 0.1, 0.2, 0.0]


def test_per_sample_results_are_split_by_work_item():
    """integrate_sample_norms and integrate_samples_batch hand back one array per work item, in
    work order, cut by the items' sample counts."""
    exp = models.eg_discrete_bath(n_tau=8)
    dev = _device(exp)
    works = [Work(0, 0.0, 0.1, 0.2, 0, n, 64) for n in (5, 1, 7)]
    _, norms = dev.integrate_sample_norms(works)
    assert [list(x) for x in norms] == [[0, 1, 2, 3, 4], [5], [6, 7, 8, 9, 10, 11, 12]]
    rs = dev.lib.rs
    _, samples = dev.integrate_samples_batch(works)
    assert [x.shape for x in samples] == [(5, rs), (1, rs), (7, rs)]
    assert samples[1][0, 0] == 5 * rs and samples[2][-1, -1] == 13 * rs - 1
