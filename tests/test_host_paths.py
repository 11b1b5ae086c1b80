"""Host-side result handling of qiw.device.Device, without a GPU: the C library is replaced by a
stand-in that writes a deterministic result buffer, so the unpacking, the packed layout and
the correlator's trace extraction are checked against each other."""
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
