"""The host planner's merged-DAG programs, executed on the CPU, against the oracle's
reference-style tree traversal (no GPU involved)."""
import numpy as np
import pytest

import oracle as orc
import planexec as pe
from qiw import _lib, models
from qiw.diagrammatics import get_topologies_at_order

REL = 1e-13


def _case(exp, kind, order, npa, times, N, budget=8192, corr=None):
    pk = _lib.PackedProblem(exp)
    ob = orc.OracleProblem(exp)
    if kind == _lib.QIW_GROUP_BARE:
        tops, okind = get_topologies_at_order(order), "bare"
    elif kind == _lib.QIW_GROUP_BOLD:
        tops, okind = get_topologies_at_order(order, npa if order else None), "bold"
    else:
        tops = get_topologies_at_order(order, npa, with_external_arc=True) if order else get_topologies_at_order(0)
        okind = "corr"
    hp = pe.HostPlan(pk, kind, order, npa, tops, corr=pk.corr_ops[corr] if corr is not None else None,
                     arena_budget=budget)
    got = pe.execute(hp, exp, pk, pe.p_tables(exp), *times, N)
    want = ob.integrate(okind, order, npa, [(t.pairs, t.parity) for t in tops], *times, N, corr=corr)
    scale = max(np.abs(w).max() for w in want)
    err = max(np.abs(a - b).max() for a, b in zip(got, want))
    return (err / scale if scale > 0 else err), hp


@pytest.mark.parametrize("kind,order,npa", [
    (_lib.QIW_GROUP_BARE, 1, 0), (_lib.QIW_GROUP_BARE, 3, 0),
    (_lib.QIW_GROUP_BOLD, 0, 0), (_lib.QIW_GROUP_BOLD, 1, 1), (_lib.QIW_GROUP_BOLD, 2, 3),
    (_lib.QIW_GROUP_BOLD, 3, 3), (_lib.QIW_GROUP_BOLD, 4, 1), (_lib.QIW_GROUP_BOLD, 4, 7),
    (_lib.QIW_GROUP_BOLD, 5, 1), (_lib.QIW_GROUP_BOLD, 5, 9), (_lib.QIW_GROUP_BARE, 5, 0),
])
def test_anderson_groups(kind, order, npa):
    exp = models.anderson(n_tau=30)
    g = exp.grid
    times = (g.tau(0), 0.0, g.tau(1)) if kind == _lib.QIW_GROUP_BARE else (g.tau(0), g.tau(11), g.tau(12))
    rel, hp = _case(exp, kind, order, npa, times, 64)
    assert rel < REL
    assert hp.flops < hp.tree_flops


@pytest.mark.parametrize("kind,order,npa", [
    (_lib.QIW_GROUP_BARE, 2, 0), (_lib.QIW_GROUP_BOLD, 2, 2), (_lib.QIW_GROUP_BOLD, 3, 1),
])
def test_eg_groups(kind, order, npa):
    exp = models.eg_discrete_bath(n_tau=24)
    g = exp.grid
    times = (g.tau(0), 0.0, g.tau(1)) if kind == _lib.QIW_GROUP_BARE else (g.tau(0), g.tau(9), g.tau(10))
    rel, _ = _case(exp, kind, order, npa, times, 16)
    assert rel < REL


@pytest.mark.parametrize("order,npa", [(0, 0), (1, 1), (2, 1), (3, 4)])
def test_correlator_groups(order, npa):
    exp = models.anderson(n_tau=30, corr=True)
    g = exp.grid
    for c in range(3):
        rel, _ = _case(exp, _lib.QIW_GROUP_CORRELATOR, order, npa, (g.tau(0), g.tau(13), g.tau(29)), 32, corr=c)
        assert rel < REL


def test_spline_delta_group():
    exp = models.single_level(n_tau=20, spline=True)
    g = exp.grid
    rel, _ = _case(exp, _lib.QIW_GROUP_BOLD, 3, 2, (g.tau(0), g.tau(7), g.tau(8)), 64)
    assert rel < REL


def test_budget_split_gives_same_result():
    """A tight working-set budget splits the roots into batches (less merging) -- same sum."""
    exp = models.eg_discrete_bath(n_tau=24)
    g = exp.grid
    t = (g.tau(0), g.tau(9), g.tau(10))
    rel_a, hp_a = _case(exp, _lib.QIW_GROUP_BOLD, 3, 3, t, 8, budget=8192)
    budget = hp_a.arena // 2
    rel_b, hp_b = _case(exp, _lib.QIW_GROUP_BOLD, 3, 3, t, 8, budget=budget)
    assert rel_a < REL and rel_b < REL
    assert hp_b.batches > hp_a.batches
    assert hp_b.arena <= budget < hp_a.arena


def test_instruction_cap_split_gives_same_result(monkeypatch):
    """Split-batch programs (batches capped at a number of instructions, the FP32 launches of
    few waves) sum to the same result, with more batches and none above the cap."""
    exp = models.eg_discrete_bath(n_tau=24)
    g = exp.grid
    t = (g.tau(0), g.tau(9), g.tau(10))
    rel_a, hp_a = _case(exp, _lib.QIW_GROUP_BOLD, 4, 4, t, 4)
    cap = 9000
    monkeypatch.setenv("QIW_MAX_BATCH_INSTRS", str(cap))
    rel_b, hp_b = _case(exp, _lib.QIW_GROUP_BOLD, 4, 4, t, 4)
    assert rel_a < REL and rel_b < REL
    assert hp_b.batches > hp_a.batches and len(hp_b.ins) > len(hp_a.ins)
    import ctypes as C
    lib = pe.plan_lib()
    lib.qiwp_batch_begin.restype = C.c_int
    pk = _lib.PackedProblem(exp)
    gd, keep = _lib.pack_group(_lib.QIW_GROUP_BOLD, 4, 4, get_topologies_at_order(4, 4))
    bb = np.zeros(1024, np.int32)
    pd = pk.desc()
    n = lib.qiwp_batch_begin(C.byref(pd), C.byref(gd), C.c_int64(8192), bb.ctypes.data_as(C.c_void_p), bb.size)
    assert n == int(hp_b.batches) + 1 and bb[n - 1] == len(hp_b.ins)
    assert np.diff(bb[:n]).max() <= cap


def test_packing_limits_are_reported():
    """The planner packs positions and pair indices into bytes: a problem with more than 256
    interaction pairs is refused with QIW_ERR_UNSUPPORTED instead of being planned wrongly."""
    from qiw.expansion import Expansion
    base = models.anderson(n_tau=8)
    pairs = list(base.pairs) * 65   # 260 pairs
    exp = Expansion(base.ed, base.grid, pairs)
    pk = _lib.PackedProblem(exp)
    with pytest.raises(_lib.QiwError) as ei:
        pe.HostPlan(pk, _lib.QIW_GROUP_BOLD, 1, 1, get_topologies_at_order(1, 1))
    assert ei.value.code == _lib.QIW_ERR_UNSUPPORTED
    exp = Expansion(base.ed, base.grid, list(base.pairs) * 64)   # 256 pairs: planned
    assert pe.HostPlan(_lib.PackedProblem(exp), _lib.QIW_GROUP_BOLD, 1, 1,
                       get_topologies_at_order(1, 1)).batches > 0


def test_offdiagonal_leaf_is_reported():
    """A block off-diagonal leaf raises, like the reference's assertion (topology_eval.jl:462)."""
    from qiw import operators as op
    from qiw.ed import EDCore
    from qiw.expansion import Expansion, InteractionPair
    from qiw.gf import ImaginaryTimeGrid, DeltaDOS, gf_from_dos, ph_conj
    H = 0.3 * op.n("a") - 0.2 * op.n("b")
    soi = op.SetOfIndices([["a"], ["b"]])
    ed = EDCore(H, soi)
    grid = ImaginaryTimeGrid(5.0, 8)
    D = gf_from_dos(DeltaDOS.make([0.1]), grid)
    # a pair moving an electron a -> b: sectors do not close on themselves
    exp = Expansion(ed, grid, [InteractionPair(op.c_dag("b"), op.c("a"), D),
                               InteractionPair(op.c("a"), op.c_dag("b"), ph_conj(D))])
    pk = _lib.PackedProblem(exp)
    tops = get_topologies_at_order(1, 1)
    with pytest.raises(_lib.QiwError) as ei:
        pe.HostPlan(pk, _lib.QIW_GROUP_BOLD, 1, 1, tops)
    assert ei.value.code == _lib.QIW_ERR_OFFDIAG


@pytest.mark.parametrize("name,order", [("anderson", 1), ("anderson", 2), ("anderson", 3), ("eg", 2), ("eg", 3)])
def test_self_energy_groups(name, order):
    """diff_inchworm! self-energy groups: PairNodes at t_i and t_f (src/inchworm.jl:560-566)."""
    exp = models.anderson(n_tau=30) if name == "anderson" else models.eg_discrete_bath(n_tau=30)
    g = exp.grid
    pk = _lib.PackedProblem(exp)
    tops = get_topologies_at_order(order, 1)
    hp = pe.HostPlan(pk, _lib.QIW_GROUP_SIGMA, order, 1, tops)
    assert hp.D == 2 * order - 2 and hp.n_fixed == 4
    t = (g.tau(0), 0.0, g.tau(13))
    got = pe.execute(hp, exp, pk, pe.p_tables(exp), *t, 64)
    want = orc.OracleProblem(exp).integrate("sigma", order, 1, [(x.pairs, x.parity) for x in tops], *t, 64)
    scale = max(np.abs(w).max() for w in want)
    assert max(np.abs(a - b).max() for a, b in zip(got, want)) <= REL * scale


def test_batch_flops_add_up_to_the_plan():
    """Per-batch flop counts (the load-balancing cost of a tile) sum, with the per-sample P and
    Delta lookups, to the plan's flops per sample."""
    import ctypes as C
    exp = models.eg_discrete_bath(n_tau=30)
    pk = _lib.PackedProblem(exp)
    pd = pk.desc()
    lib = pe.plan_lib()
    lib.qiwp_batch_flops.restype = C.c_int
    lib.qiwp_batch_flops.argtypes = [C.POINTER(_lib.ProblemDesc), C.POINTER(_lib.GroupDesc), C.c_int64,
                                     C.c_void_p, C.c_int]
    for order, npa in [(2, 2), (3, 3), (4, 4)]:
        tops = get_topologies_at_order(order, npa)
        gd, keep = _lib.pack_group(_lib.QIW_GROUP_BOLD, order, npa, tops)
        out = np.zeros(4096)
        n = lib.qiwp_batch_flops(C.byref(pd), C.byref(gd), 8192, out.ctypes.data, out.size)
        hp = pe.HostPlan(pk, _lib.QIW_GROUP_BOLD, order, npa, tops)
        assert n == int(hp.batches) and np.all(out[:n] > 0)
        dims = np.array(exp.dims)
        lookups = sum(3.0 * dims[int(j["s"])] ** 2 for j in hp.pm) + 3.0 * len(hp.wj)
        assert abs(out[:n].sum() + lookups - hp.flops) <= 1e-9 * hp.flops


def test_reference_topology_eval_fixture():
    """The reference's own TopologyEvaluator values (test/topology_eval.h5, test/topology_eval.jl:
    53-140: single level, order 3, n_pts_after = 1, 100 explicit time sets) against this
    planner's program at the same times.

    The fixture's Delta and P live on a two-time FullTimeGrid; its reversed Delta is
    Delta[t2, t1] without the sign test/dimers.jl applies, i.e. -Delta(beta - tau) here.  Where
    two integrated times fall into one tau cell, Keldysh.jl interpolates the two-time grid across
    its diagonal (a rule this build cannot inspect) and values differ by up to a factor ~8, so
    the pin is on the samples whose integrated times occupy distinct cells: there the two
    interpolation rules agree to 1e-3 (2e-3 asserted), with the phase (-i)^11 = i of 8 P and
    3 Delta factors.  With one orbital only topology ((1,4),(2,5),(3,6)) has configurations
    (the planner emits empty programs for the other three), so it is that topology, its parity
    and its configuration products that the fixture pins; a flipped parity fails the test."""
    import json, os
    from qiw import operators as op
    from qiw.ed import EDCore
    from qiw.expansion import Expansion, InteractionPair
    from qiw.gf import ImaginaryTimeGF, ImaginaryTimeGrid, DeltaDOS, gf_from_dos, ph_conj
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "topology_eval_h5.json")))
    md = gold["model"]
    beta, n_tau = md["beta"], md["n_tau"]
    ed = EDCore(-md["mu"] * op.n("0"), op.SetOfIndices([["0"]]))
    grid = ImaginaryTimeGrid(beta, n_tau)
    D = md["V"] ** 2 * gf_from_dos(DeltaDOS.make([md["eps"]]), grid)
    Dr = ph_conj(D)
    Dr = ImaginaryTimeGF(Dr.grid, Dr.norb, Dr.xi == -1, -Dr.data)
    exp = Expansion(ed, grid, [InteractionPair(op.c_dag("0"), op.c("0"), D),
                               InteractionPair(op.c("0"), op.c_dag("0"), Dr)])
    pk = _lib.PackedProblem(exp)
    hp = pe.HostPlan(pk, _lib.QIW_GROUP_BOLD, md["order"], md["n_pts_after"],
                     get_topologies_at_order(md["order"], md["n_pts_after"]))
    h = grid.step
    x0, xw, xf = 0.0, md["tau_index_w"] * h, md["tau_index_f"] * h
    x1 = np.array(gold["x1_list"])
    xs = np.array(gold["xs_list"])
    Ns = len(x1)
    u = np.vstack([xw + (xf - xw) * x1[None, :], x0 + (xw - x0) * xs])   # test/topology_eval.jl:108-113
    tm = np.zeros((hp.n_nodes, Ns))
    for p_, ts in zip(hp.fixed_pos, hp.fixed_time):
        tm[p_] = (x0, xw, xf)[ts]
    for j in range(hp.D):
        tm[hp.var_pos[j]] = u[j]
    R = pe.run_program(hp, exp, pk, pe.p_tables(exp), tm)
    want = np.array([np.array(v["re"]) + 1j * np.array(v["im"]) for v in gold["values"]]).T   # [Ns][2]
    got = 1j * R[:2].T
    distinct = np.array([len(set(np.floor(u[:, i] / h).astype(int))) == hp.D for i in range(Ns)])
    assert distinct.sum() >= 10
    rel = np.abs(got - want).max(axis=1) / np.abs(want).max(axis=1)
    assert rel[distinct].max() < 2e-3
    assert np.median(rel) < 2e-3   # most samples agree even with shared cells


def _reads(I):
    """Arena ranges an instruction reads (start, length), as the kernel's interpreter does."""
    op, r, k, c = int(I["op"]), int(I["rows"]), int(I["inner"]), int(I["cols"])
    src, a, w = int(I["src"]), int(I["a"]), int(I["w"])
    out = [(w, 1)] if w >= 0 else []
    if op == 3:
        out += [(a, r * r), (src, r * c)]
    elif op == 5:
        out += [(src, k * c)] + ([(int(I["dst"]), r * c)] if int(I["acc"]) else [])
    elif op == 6:
        out += [(src, r * c)] + ([(int(I["dst"]), r * c)] if int(I["acc"]) else [])
    elif op == 7:
        out += [(src, r * c)]
    return out


@pytest.mark.parametrize("model,order,npa", [("eg", 3, 2), ("eg", 4, 4), ("t2g", 2, 2), ("anderson", 3, 3)])
def test_register_product_flags_are_consistent(model, order, npa):
    """Planner flags for the FP32 interpreter's register-held products: an edge marked 'source
    in registers' (bit 2) follows its node's P multiply marked 'keep' (bit 3) with no other
    instruction in between, has that product's shape, and reads nothing of the arena copy; a
    product marked 'no store' (bit 4) is read from the arena by no instruction before its slot
    is written again.  Only blocks of dimension 1, 2, 4 are marked; 1x1 programs are not."""
    exp = {"eg": lambda: models.eg_discrete_bath(n_tau=24), "t2g": lambda: models.t2g_bethe(n_tau=24),
           "anderson": lambda: models.anderson(n_tau=24)}[model]()
    pk = _lib.PackedProblem(exp)
    tops = get_topologies_at_order(order, npa)
    hp = pe.HostPlan(pk, _lib.QIW_GROUP_BOLD, order, npa, tops, arena_budget=20480 if model == "t2g" else 8192)
    ins = hp.ins
    flags = ins["flags"]
    keep = None   # (index, rows, cols) of the last P multiply kept in registers
    n_marked = 0
    for i, I in enumerate(ins):
        op, f = int(I["op"]), int(flags[i])
        if op == 3 and f & 8:
            keep = (i, int(I["rows"]), int(I["cols"]))
            assert int(I["rows"]) in (1, 2, 4) and int(I["cols"]) in (1, 2, 4)
            n_marked += 1
            if f & 16:   # no instruction reads the product's slot before it is written again
                lo, n = int(I["dst"]), int(I["rows"]) * int(I["cols"])
                for J in ins[i + 1:]:
                    fj = int(J["flags"])
                    if not (int(J["op"]) in (5, 6) and fj & 4):
                        assert all(s + m <= lo or s >= lo + n for s, m in _reads(J))
                    if int(J["op"]) in (1, 2, 3, 4, 5, 6, 8, 9) and int(J["dst"]) < lo + n and \
                            int(J["dst"]) + int(J["rows"]) * max(int(J["cols"]), 1) > lo and not int(J["acc"]):
                        break
            continue
        if op in (5, 6) and f & 4:
            assert keep is not None
            assert int(I["inner" if op == 5 else "rows"]) == keep[1] and int(I["cols"]) == keep[2]
            assert int(I["rows"]) in (1, 2, 4)
            continue
        keep = None
    if model == "eg":
        assert n_marked > 0
    if model == "anderson":
        assert n_marked == 0   # 1x1 programs fuse differently (PMAXPY)
