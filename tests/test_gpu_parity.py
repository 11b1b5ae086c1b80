"""CUDA path (through the C ABI) against the CPU oracle on the same seeded inputs.

Tolerance: the plain FP64 path must agree with the oracle to 1e-12 relative (max-abs error
over the group's result blocks / max-abs of the oracle's blocks); the FP32 chain-product path
to 1e-4.
"""
import numpy as np
import pytest

import oracle as orc
from qiw import _lib, models
from qiw.device import Work
from qiw.diagrammatics import get_topologies_at_order

pytestmark = pytest.mark.gpu

REL64 = 1e-12
REL32 = 1e-4


def _rel(got, want):
    scale = max(np.abs(w).max() for w in want)
    err = max(np.abs(a - b).max() for a, b in zip(got, want))
    return err / scale if scale > 0 else err


def _tops(kind, order, npa):
    if kind == _lib.QIW_GROUP_BARE:
        return get_topologies_at_order(order)
    if order == 0:
        return get_topologies_at_order(0)
    return get_topologies_at_order(order, npa, with_external_arc=(kind == _lib.QIW_GROUP_CORRELATOR))


def _okind(kind):
    return {_lib.QIW_GROUP_BARE: "bare", _lib.QIW_GROUP_BOLD: "bold", _lib.QIW_GROUP_CORRELATOR: "corr"}[kind]


CASES = [
    ("anderson", _lib.QIW_GROUP_BARE, 2, 0), ("anderson", _lib.QIW_GROUP_BARE, 4, 0),
    ("anderson", _lib.QIW_GROUP_BOLD, 0, 0), ("anderson", _lib.QIW_GROUP_BOLD, 1, 1),
    ("anderson", _lib.QIW_GROUP_BOLD, 3, 2), ("anderson", _lib.QIW_GROUP_BOLD, 4, 4),
    ("anderson", _lib.QIW_GROUP_CORRELATOR, 2, 1), ("anderson", _lib.QIW_GROUP_CORRELATOR, 3, 5),
    ("eg", _lib.QIW_GROUP_BARE, 2, 0), ("eg", _lib.QIW_GROUP_BOLD, 2, 2), ("eg", _lib.QIW_GROUP_BOLD, 3, 3),
    ("single", _lib.QIW_GROUP_BOLD, 3, 1),
]


def _model(name):
    if name == "anderson":
        return models.anderson(n_tau=40, corr=True)
    if name == "eg":
        return models.eg_discrete_bath(n_tau=40)
    return models.single_level(n_tau=20, spline=True)


@pytest.mark.parametrize("name,kind,order,npa", CASES)
def test_group_fp64_matches_oracle(device, name, kind, order, npa):
    exp = _model(name)
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    tops = _tops(kind, order, npa)
    corr = 0 if kind == _lib.QIW_GROUP_CORRELATOR else None
    gid = device.create_group(kind, order, npa, tops, corr)
    if kind == _lib.QIW_GROUP_BARE:
        t = (g.tau(0), 0.0, g.tau(1))
    elif kind == _lib.QIW_GROUP_BOLD:
        t = (g.tau(0), g.tau(17), g.tau(18))
    else:
        t = (g.tau(0), g.tau(9), g.tau(g.n_tau - 1))
    N = 128
    got = device.integrate([Work(gid, *t, 0, N, N)])[0]
    want = orc.OracleProblem(exp).integrate(_okind(kind), order, npa, [(x.pairs, x.parity) for x in tops],
                                            *t, N, corr=corr)
    assert _rel(got, want) < REL64
    got32 = device.integrate([Work(gid, *t, 0, N, N)], precision=_lib.QIW_PREC_FP32)[0]
    assert _rel(got32, want) < REL32


def test_ragged_ranges_and_rank_split(device):
    exp = models.anderson(n_tau=30)
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    tops = get_topologies_at_order(3, 3)
    gid = device.create_group(_lib.QIW_GROUP_BOLD, 3, 3, tops)
    t = (g.tau(0), g.tau(10), g.tau(11))
    ob = orc.OracleProblem(exp)
    tl = [(x.pairs, x.parity) for x in tops]
    for N in (1, 3, 100, 257):
        got = device.integrate([Work(gid, *t, 0, N, N)])[0]
        assert _rel(got, ob.integrate("bold", 3, 3, tl, *t, N)) < REL64
    # three "ranks" with rank_sub_range chunks, one launch, summed like all_reduce!
    N = 512
    chunks = [171, 171, 170]
    starts = [0, 171, 342]
    parts = device.integrate([Work(gid, *t, s, c, N) for s, c in zip(starts, chunks)])
    tot = [sum(p[s] for p in parts) for s in range(len(parts[0]))]
    assert _rel(tot, ob.integrate("bold", 3, 3, tl, *t, N, n_ranks=3)) < REL64


def test_zero_samples_and_errors(device):
    exp = models.anderson(n_tau=16)
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    gid = device.create_group(_lib.QIW_GROUP_BOLD, 1, 1, get_topologies_at_order(1, 1))
    g = exp.grid
    got = device.integrate([Work(gid, g.tau(0), g.tau(3), g.tau(4), 0, 0, 16)])[0]
    assert all(np.all(b == 0) for b in got)
    with pytest.raises(_lib.QiwError) as ei:
        device.integrate([Work(gid + 1000, 0.0, 0.1, 0.2, 0, 8, 8)])
    assert ei.value.code == _lib.QIW_ERR_ARG
    with pytest.raises(_lib.QiwError):
        device.integrate([Work(gid, 0.5, 0.1, 0.2, 0, 8, 8)])   # t_i > t_w


def test_complex_phase_input_is_rejected(device):
    exp = models.anderson(n_tau=16)
    device.set_problem(exp)
    P = [p.copy() for p in exp.P]
    P[0].data = P[0].data + 1e-3   # real part: not of the imaginary-branch form -i * real
    device.set_ppgf(P)
    gid = device.create_group(_lib.QIW_GROUP_BOLD, 1, 1, get_topologies_at_order(1, 1))
    with pytest.raises(_lib.QiwError) as ei:
        device.integrate([Work(gid, 0.0, 1.0, 1.5, 0, 8, 8)])
    assert ei.value.code == _lib.QIW_ERR_UNSUPPORTED


def test_rerun_is_bit_identical(device):
    exp = models.eg_discrete_bath(n_tau=32)
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    gid = device.create_group(_lib.QIW_GROUP_BOLD, 3, 2, get_topologies_at_order(3, 2))
    w = [Work(gid, g.tau(0), g.tau(12), g.tau(13), 0, 1000, 1024)]
    a = device.integrate(w)[0]
    b = device.integrate(w)[0]
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


def test_inchworm_loop_matches_oracle(device):
    from qiw.inchworm import inchworm
    exp = models.anderson(n_tau=24)
    exp_o = models.anderson(n_tau=24)
    inchworm(exp, range(0, 4), range(0, 4), 64, dev=device)
    pb = orc.inchworm(exp_o, range(0, 4), range(0, 4), 64)
    for s in range(len(exp.P)):
        a, b = exp.P[s].data, pb.P_data[s]
        assert np.abs(a - b).max() <= 1e-11 * np.abs(b).max()


def test_golden_inchworm_h5_through_gpu(device):
    """The reference's own fixture (test/inchworm.h5, test/inchworm.jl:180-212) on the GPU path."""
    import json, os
    from qiw import operators as op
    from qiw.inchworm import inchworm, correlator_2p
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "inchworm_h5.json")))
    exp = models.single_level()
    inchworm(exp, range(0, 4), range(0, 3), 2 ** 8, dev=device)
    for s in range(2):
        want = np.array(gold["P"][s]["re"]) + 1j * np.array(gold["P"][s]["im"])
        got = exp.P[s].data[:, 0, 0]
        assert np.linalg.norm(got - want) <= 5e-8 * np.linalg.norm(want)
    exp.add_corr_operators((op.c("0"), op.c_dag("0")))
    g = -correlator_2p(exp, range(0, 4), 2 ** 8, dev=device)[0]
    want = np.array(gold["g"]["re"]) + 1j * np.array(gold["g"]["im"])
    assert np.linalg.norm(g - want) <= 1e-6 * np.linalg.norm(want)


def test_correlator_matches_oracle(device):
    from qiw.inchworm import correlator_2p
    exp = models.anderson(n_tau=20, corr=True)
    device.set_problem(exp)
    got = correlator_2p(exp, range(0, 3), 64, dev=device)
    pb = orc.OracleProblem(exp)
    want = orc.correlator_2p(pb, range(0, 3), 64)
    for a, b in zip(got, want):
        assert np.abs(a - b).max() <= 1e-11 * np.abs(b).max()


def test_fp32_path_errors_are_stated_and_small(device):
    """FP32 chain products with FP64 accumulation: max |P_FP32 - P_FP64| and the G(tau)
    difference on a full inchworm! + correlator_2p run with the same Sobol points."""
    from qiw import ppgf
    from qiw.inchworm import inchworm, correlator_2p
    res = {}
    for prec in (_lib.QIW_PREC_FP64, _lib.QIW_PREC_FP32):
        exp = models.anderson(n_tau=24, corr=True)
        inchworm(exp, range(0, 4), range(0, 4), 256, dev=device, precision=prec)
        ppgf.normalize_beta(exp.P, exp.grid.beta)
        g = correlator_2p(exp, range(0, 3), 256, dev=device, precision=prec)
        res[prec] = ([P_s.data.copy() for P_s in exp.P], np.array(g))
    dP = max(np.abs(a - b).max() for a, b in zip(res[0][0], res[1][0]))
    dG = np.abs(res[0][1] - res[1][1]).max()
    print(f"FP32 vs FP64: max|dP| = {dP:.2e}, max|dG| = {dG:.2e}")
    assert dP < 1e-5 and dG < 1e-5


T2G_CASES = [(_lib.QIW_GROUP_BOLD, 1, 1, 64), (_lib.QIW_GROUP_BOLD, 2, 2, 64), (_lib.QIW_GROUP_BOLD, 3, 1, 12),
             (_lib.QIW_GROUP_BOLD, 3, 3, 12), (_lib.QIW_GROUP_CORRELATOR, 2, 2, 32),
             (_lib.QIW_GROUP_CORRELATOR, 3, 3, 8)]


@pytest.mark.parametrize("kind,order,npa,N", T2G_CASES)
def test_t2g_groups_match_oracle(device, kind, order, npa, N):
    """Three-orbital t2g model: sector blocks up to 9x9, order-3 groups on the largest arena."""
    exp = models.t2g_bethe(n_tau=64, corr=True)
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    tops = _tops(kind, order, npa)
    corr = 1 if kind == _lib.QIW_GROUP_CORRELATOR else None
    gid = device.create_group(kind, order, npa, tops, corr)
    t = (g.tau(0), g.tau(40), g.tau(41)) if kind == _lib.QIW_GROUP_BOLD else (g.tau(0), g.tau(23), g.tau(63))
    got = device.integrate([Work(gid, *t, 0, N, N)])[0]
    want = orc.OracleProblem(exp).integrate(_okind(kind), order, npa, [(x.pairs, x.parity) for x in tops],
                                            *t, N, corr=corr)
    assert _rel(got, want) < REL64
    got32 = device.integrate([Work(gid, *t, 0, N, N)], precision=_lib.QIW_PREC_FP32)[0]
    assert _rel(got32, want) < REL32
    # operator multiplies of 9-wide blocks on tensor cores (3xTF32): the same FP32 bound
    got_tc = device.integrate([Work(gid, *t, 0, N, N)], precision=_lib.QIW_PREC_FP32_TC)[0]
    assert _rel(got_tc, want) < REL32


@pytest.mark.parametrize("N", [16, 45])
def test_t2g_tensor_core_operator_multiplies_match_fp32(device, N):
    """QIW_PREC_FP32_TC against QIW_PREC_FP32 and the oracle on the heaviest t2g order-3 group,
    with a sample count that leaves part of the last warp without a sample (those lanes run the
    program for the warp's tensor-core multiplies and contribute nothing)."""
    exp = models.t2g_bethe(n_tau=64)
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    tops = get_topologies_at_order(3, 3)
    gid = device.create_group(_lib.QIW_GROUP_BOLD, 3, 3, tops)
    t = (g.tau(0), g.tau(40), g.tau(41))
    want = orc.OracleProblem(exp).integrate("bold", 3, 3, [(x.pairs, x.parity) for x in tops], *t, N)
    got32 = device.integrate([Work(gid, *t, 0, N, N)], precision=_lib.QIW_PREC_FP32)[0]
    got_tc = device.integrate([Work(gid, *t, 0, N, N)], precision=_lib.QIW_PREC_FP32_TC)[0]
    rel_tc = _rel(got_tc, want)
    print(f"t2g order 3 N={N}: FP32 {_rel(got32, want):.2e}, FP32 + tensor cores {rel_tc:.2e}")
    assert rel_tc < REL32
    assert _rel(got_tc, got32) < REL32


@pytest.mark.parametrize("name,order", [("anderson", 1), ("anderson", 3), ("eg", 2)])
def test_bare_domain_maps_match_oracle(device, name, order):
    """SortTransform and ExpModelFunctionTransform on bare groups: kernel against the oracle."""
    exp = _model(name)
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    tops = _tops(_lib.QIW_GROUP_BARE, order, 0)
    gid = device.create_group(_lib.QIW_GROUP_BARE, order, 0, tops)
    tl = [(x.pairs, x.parity) for x in tops]
    ob = orc.OracleProblem(exp)
    t_f = g.tau(5)
    N = 256
    decay = t_f / (2 * order)
    for tr, kw, t_w in [(_lib.QIW_TRANSFORM_SORT, dict(transform="sort"), 0.0),
                        (_lib.QIW_TRANSFORM_EXPMODEL, dict(transform="expmodel", decay=decay), decay)]:
        w = [Work(gid, 0.0, t_w, t_f, 0, N, N, transform=tr)]
        want = ob.integrate("bare", order, 0, tl, 0.0, 0.0, t_f, N, **kw)
        assert _rel(device.integrate(w)[0], want) < REL64, tr
        assert _rel(device.integrate(w, precision=_lib.QIW_PREC_FP32)[0], want) < REL32, tr


def test_domain_map_arguments_are_checked(device):
    exp = _model("anderson")
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    bare = device.create_group(_lib.QIW_GROUP_BARE, 1, 0, _tops(_lib.QIW_GROUP_BARE, 1, 0))
    bold = device.create_group(_lib.QIW_GROUP_BOLD, 1, 1, _tops(_lib.QIW_GROUP_BOLD, 1, 1))
    bad = [Work(bold, g.tau(0), g.tau(3), g.tau(4), 0, 64, 64, transform=_lib.QIW_TRANSFORM_SORT),
           Work(bare, g.tau(1), 0.5, g.tau(4), 0, 64, 64, transform=_lib.QIW_TRANSFORM_EXPMODEL),
           Work(bare, 0.0, 0.0, g.tau(4), 0, 64, 64, transform=_lib.QIW_TRANSFORM_EXPMODEL),
           Work(bare, 0.0, 0.0, g.tau(4), 0, 64, 64, transform=7)]
    for w in bad:
        with pytest.raises(_lib.QiwError) as e:
            device.integrate([w])
        assert e.value.code == _lib.QIW_ERR_ARG


@pytest.mark.parametrize("name,order", [("anderson", 1), ("anderson", 3), ("eg", 2), ("eg", 3)])
def test_self_energy_groups_match_oracle(device, name, order):
    exp = _model(name)
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    tops = get_topologies_at_order(order, 1)
    gid = device.create_group(_lib.QIW_GROUP_SIGMA, order, 1, tops)
    t = (g.tau(0), 0.0, g.tau(17))
    N = 128
    want = orc.OracleProblem(exp).integrate("sigma", order, 1, [(x.pairs, x.parity) for x in tops], *t, N)
    assert _rel(device.integrate([Work(gid, *t, 0, N, N)])[0], want) < REL64
    assert _rel(device.integrate([Work(gid, *t, 0, N, N)], precision=_lib.QIW_PREC_FP32)[0], want) < REL32


def test_diff_inchworm_loop_matches_oracle(device):
    from qiw.inchworm import diff_inchworm
    exp = models.anderson(n_tau=16)
    diff_inchworm(exp, range(0, 4), 64, dev=device)
    pb, _ = orc.diff_inchworm(models.anderson(n_tau=16), range(0, 4), 64)
    for s in range(len(exp.P)):
        assert np.abs(exp.P[s].data - pb.P_data[s]).max() <= 1e-11 * np.abs(pb.P_data[s]).max()


def test_golden_diff_inchworm_h5_through_gpu(device):
    """The reference's fixture (test/inchworm.h5 /diff_inchworm/P, test/inchworm.jl:214-239)."""
    import json, os
    from qiw.inchworm import diff_inchworm
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "inchworm_h5.json")))
    exp = models.single_level()
    diff_inchworm(exp, range(0, 4), 2 ** 8, dev=device)
    for s in range(2):
        want = np.array(gold["diff_P"][s]["re"]) + 1j * np.array(gold["diff_P"][s]["im"])
        got = exp.P[s].data[:, 0, 0]
        assert np.linalg.norm(got - want) <= 5e-8 * np.linalg.norm(want)


def test_readme_anderson_output_through_gpu(device):
    """The reference README's workflow (README.md:51-125: Anderson model, inchworm! orders 0:4,
    bare 0:4, N = 2^10, n_tau = 200) against its printed rho (README.md:204).

    The printed Z = 22.515 (README.md:203) is not reproduced by the reference's current
    inchworm!: after every step it rescales P so that max_s,i -Im P_s,ii(tau_f) = 1
    (src/inchworm.jl:489 with src/ppgf.jl:646-654), so at tau_f = beta the un-normalized
    Z = sum_s Tr[i P_s(beta)] equals 1 / max_s rho_s exactly.  The test asserts that identity."""
    import json, os
    from qiw import ppgf
    from qiw.inchworm import inchworm
    ra = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "readme_anderson.json")))
    exp = models.anderson()
    inchworm(exp, range(0, 5), range(0, 5), 2 ** 10, dev=device)
    Z = ppgf.partition_function(exp.P)
    ppgf.normalize_beta(exp.P, exp.grid.beta)
    rho = [float(np.real(m[0, 0])) for m in ppgf.density_matrix(exp.P)]
    print(f"README run: Z = {Z.real:.10f}, rho = {rho} (README {ra['rho']})")
    assert abs(Z.imag) < 1e-12
    assert abs(Z.real * max(rho) - 1.0) < 1e-10
    assert np.allclose(rho, ra["rho"], atol=1e-4)


def test_plan_cache_reuses_plans_across_problems(device):
    """qiw_plan_cache_*: a second solve on the same operators (new Delta, beta, grid) plans no
    group again and gives the same P as a solve with an empty cache; operators with other
    block values (eg Kanamori with another J rotates the eigenbasis) are planned anew; a
    batch reuses the plans of the host-driven loop."""
    from qiw.inchworm import inchworm
    device.plan_cache_clear()
    a = models.anderson(n_tau=16, V=0.5)
    inchworm(a, range(0, 4), range(0, 4), 64, dev=device)
    i1 = device.plan_cache_info()
    b = models.anderson(n_tau=20, V=0.6, beta=5.0)
    inchworm(b, range(0, 4), range(0, 4), 64, dev=device)
    i2 = device.plan_cache_info()
    assert i1["entries"] > 0 and i2["entries"] == i1["entries"]
    assert i2["hits"] - i1["hits"] >= i1["entries"]
    device.plan_cache_clear()
    assert device.plan_cache_info()["entries"] == 0
    c = models.anderson(n_tau=20, V=0.6, beta=5.0)
    inchworm(c, range(0, 4), range(0, 4), 64, dev=device)
    for s in range(len(b.P)):
        assert np.array_equal(b.P[s].data, c.P[s].data)
    device.plan_cache_clear()
    inchworm(models.eg_discrete_bath(n_tau=8, J=0.2), range(0, 3), range(0, 3), 64, dev=device)
    e1 = device.plan_cache_info()
    inchworm(models.eg_discrete_bath(n_tau=8, J=0.3), range(0, 3), range(0, 3), 64, dev=device)
    e2 = device.plan_cache_info()
    assert e2["entries"] > e1["entries"]
    from qiw.batch import inchworm_batch
    device.plan_cache_clear()
    h = models.anderson(n_tau=20, V=0.6, beta=5.0)
    inchworm(h, range(0, 4), range(0, 4), 64, dev=device)
    i3 = device.plan_cache_info()
    d = models.anderson(n_tau=20, V=0.6, beta=5.0)
    inchworm_batch([d], range(0, 4), range(0, 4), 64, autotune=False)
    i4 = device.plan_cache_info()
    assert i4["entries"] == i3["entries"] and i4["hits"] > i3["hits"]
    for s in range(len(h.P)):
        assert np.abs(h.P[s].data - d.P[s].data).max() <= 1e-12 * np.abs(h.P[s].data).max()


@pytest.mark.parametrize("kind,order,npa", [
    (_lib.QIW_GROUP_BOLD, 5, 1), (_lib.QIW_GROUP_BOLD, 5, 9), (_lib.QIW_GROUP_BOLD, 6, 1),
    (_lib.QIW_GROUP_BOLD, 6, 6), (_lib.QIW_GROUP_BARE, 5, 0), (_lib.QIW_GROUP_BARE, 6, 0),
])
def test_highest_orders_match_oracle(device, kind, order, npa):
    """Orders 5 and 6 (D = 10 and 12 Sobol dimensions, the largest the batched solves use; up to
    10395 bare topologies), FP64 and FP32, against the oracle."""
    exp = models.anderson(n_tau=30)
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    tops = _tops(kind, order, npa)
    gid = device.create_group(kind, order, npa, tops)
    t = (g.tau(0), 0.0, g.tau(1)) if kind == _lib.QIW_GROUP_BARE else (g.tau(0), g.tau(20), g.tau(21))
    N = 32
    want = orc.OracleProblem(exp).integrate(_okind(kind), order, npa, [(x.pairs, x.parity) for x in tops], *t, N)
    assert _rel(device.integrate([Work(gid, *t, 0, N, N)])[0], want) < REL64
    assert _rel(device.integrate([Work(gid, *t, 0, N, N)], precision=_lib.QIW_PREC_FP32)[0], want) < REL32


@pytest.mark.parametrize("npa", [4, 7])
def test_fp32_split_batch_programs_match_oracle(device, monkeypatch, npa):
    """eg order-4 groups carry split-batch programs (batches capped at 11000 / 9000
    instructions) for FP32 launches of few waves; every level agrees with the oracle at the
    FP32 tolerance, and the levels differ from each other by FP32 rounding only."""
    exp = models.eg_discrete_bath(n_tau=40)
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    g = exp.grid
    t = (g.tau(0), g.tau(20), g.tau(21))
    tops = get_topologies_at_order(4, npa)
    gid = device.create_group(_lib.QIW_GROUP_BOLD, 4, npa, tops)
    N = 48
    want = orc.OracleProblem(exp).integrate("bold", 4, npa, [(x.pairs, x.parity) for x in tops], *t, N)
    got = {}
    for level in (0, 1, 2):
        monkeypatch.setenv("QIW_SPLIT_LEVEL", str(level))
        got[level] = device.integrate([Work(gid, *t, 0, N, N)], _lib.QIW_PREC_FP32)[0]
        assert _rel(got[level], want) < REL32, level
    monkeypatch.delenv("QIW_SPLIT_LEVEL")
    assert _rel(device.integrate([Work(gid, *t, 0, N, N)], _lib.QIW_PREC_FP32)[0], want) < REL32   # chosen level
    for level in (1, 2):
        assert _rel(got[level], got[0]) < 1e-5
