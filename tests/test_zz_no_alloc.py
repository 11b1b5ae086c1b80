"""qiw_integrate_noalloc: the integration entry point that allocates no device memory.

It exists for callers that cannot call cudaMalloc while they run -- for instance code that
works inside a host framework which owns every device allocation (so the caller hands in a
buffer the framework gave it), or code that must not allocate between setup and teardown.
Its scratch is a fixed 16 MiB static device array shared by all calls; the result goes into
a device buffer the caller owns.  This test compares it, through the C ABI, with the regular
qiw_integrate on the same inputs, on two calls in a row (the second call finds the previous
call's contents in the shared array).  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from qiw import _lib, models
from qiw.device import Work
from qiw.diagrammatics import get_topologies_at_order

pytestmark = pytest.mark.gpu

REL = {_lib.QIW_PREC_FP64: 1e-12, _lib.QIW_PREC_FP32: 1e-4}


def _descs(device, works):
    descs = (_lib.WorkDesc * len(works))()
    keep = []
    for i, w in enumerate(works):
        D = 2 * device.group_info[w.group][1]
        m = np.ascontiguousarray(device.sobol(D) if D else np.zeros((1, 32), np.uint32))
        x0 = np.zeros(max(D, 1), np.uint32)
        keep += [m, x0]
        descs[i] = _lib.WorkDesc(w.group, 0, w.t_i, w.t_w, w.t_f, w.first_index, w.n_samples,
                                 w.n_total, m.ctypes.data, x0.ctypes.data)
    return descs, keep


@pytest.mark.parametrize("precision", [_lib.QIW_PREC_FP64, _lib.QIW_PREC_FP32])
def test_noalloc_matches_integrate_twice(device, precision):
    import torch
    exp = models.eg_discrete_bath(n_tau=48)
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    gids = [device.create_group(_lib.QIW_GROUP_BOLD, k, npa, get_topologies_at_order(k, npa))
            for (k, npa) in [(1, 1), (2, 2), (3, 1), (3, 4)]]
    gids.append(device.create_group(_lib.QIW_GROUP_BOLD, 0, 0, get_topologies_at_order(0)))
    rs = int(np.sum(np.array(exp.dims) ** 2))
    lib = device.lib
    for call, (n, N) in enumerate([(17, 384), (21, 256)]):
        works = [Work(gid, g.tau(0), g.tau(n), g.tau(n + 1), 0, N, N) for gid in gids]
        want = device.integrate(works, precision)
        descs, keep = _descs(device, works)
        out = torch.full((2 * rs * len(works),), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = lib.qiw_integrate_noalloc(device.h, len(works), descs, precision, C.c_void_p(out.data_ptr()))
        assert rc == _lib.QIW_OK, lib.qiw_last_error(device.h).decode()
        z = out.cpu().numpy()
        z = z[0::2] + 1j * z[1::2]
        for i, blocks in enumerate(want):
            ref = np.concatenate([b.ravel(order="F") for b in blocks])
            got = z[i * rs:(i + 1) * rs]
            scale = np.abs(ref).max()
            assert np.abs(got - ref).max() <= REL[precision] * scale, (call, i)


def test_noalloc_rejects_oversized_calls(device):
    import torch
    exp = models.anderson(n_tau=16)
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    gid = device.create_group(_lib.QIW_GROUP_BOLD, 1, 1, get_topologies_at_order(1, 1))
    g = exp.grid
    # 2^27 samples: at most 128 samples per tile (any thread setting), at least 2^20 CTAs whose
    # map and partial sums need far more than the 16 MiB array
    works = [Work(gid, g.tau(0), g.tau(3), g.tau(4), 0, 1 << 27, 1 << 27)]
    descs, keep = _descs(device, works)
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = device.lib.qiw_integrate_noalloc(device.h, 1, descs, _lib.QIW_PREC_FP64, C.c_void_p(out.data_ptr()))
    assert rc == _lib.QIW_ERR_MEMORY
    msg = device.lib.qiw_last_error(device.h).decode()
    assert "maximum" in msg
    needed = int(msg.split("needs ")[1].split(" bytes")[0])
    assert needed > 16 << 20
