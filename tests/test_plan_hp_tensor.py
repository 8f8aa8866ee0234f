"""Planner side of the tensor-core hole products and accumulations
(double-float plans with flavour bit 0x8000), on the CPU.  In every hole-product stage the tasks with
16 <= a <= 64 and at least 128 reduction rows go into groups of up to
min(8, 128 / a) tasks that share the operand A (same buffer, offset and
shape); every group's work items cover its 64-row chunks exactly once, in
ranges of the length the member tasks record (kchunk, splits); split tasks
own disjoint workspace slots; one pre-pass image per distinct A, private
within the stage and inside B_OZ; the other tasks keep their classic tiles.
Accumulations with 16 <= d <= 64 and at least 64 rows get one item per
128-row block (all terms in order, one unit each, items ordered by their
units-before count) and an image slot per term."""
import numpy as np
import pytest

from plan_emulator import ST_ACC, ST_HP, PlanView, acc_tc_eligible, hp_tc_eligible
from qutree_gb300.model import balanced_tree, config_problem, coupled_oscillators

TENSOR = 0x8000
CHUNK = 64


def kc_of(a):
    return 2 * CHUNK if (a + 7) // 8 * 8 > 32 else CHUNK  # 128 k where four level accumulators are used


def chunk_bytes(a, steps):
    ap = (a + 7) // 8 * 8
    return steps * 7 * 3 * ap * 16 * 2 + 64 * 4


def wide_leaf_problem():
    tree = balanced_tree(4, 80, 12)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=np.random.default_rng(8),
                              omega=1.0)
    return tree, sop


def problem(name):
    if name == "wide_leaves":
        return wide_leaf_problem()
    tree, sop, _ = config_problem(int(name[3:]))
    return tree, sop


@pytest.mark.parametrize("name", ["cfg0", "cfg4", "cfg1", "wide_leaves"])
@pytest.mark.parametrize("plan", [1, 2])
def test_hole_product_groups_and_items(name, plan):
    tree, sop = problem(name)
    pv = PlanView(tree, sop, flavour=plan | TENSOR, prec=1)
    T = pv.tables
    hp, hpx, tiles, groups, items, units, ranges = T[2], T[44], T[45], T[52], T[53], T[54], T[55]
    oz_bytes = int(T[56][0])
    hpw = int(T[48][0])
    n_tc = 0
    for si, (kind, t0, nt, _, _) in enumerate(T[0]):
        hti0, nhti, htu0, nhtu = (int(x) for x in ranges[si])
        if kind != ST_HP:
            assert nhti == 0 and nhtu == 0
            continue
        stage_tasks = range(t0, t0 + nt)
        eligible = {t for t in stage_tasks if hp_tc_eligible(*(int(x) for x in hp[t][6:9]))}
        its = items[hti0:hti0 + nhti]
        gids = sorted({int(g) for g, _, _, _ in its})
        seen = []
        img_of = {}
        for g in gids:
            Abuf, Aoff, bef, a, aft, n, nch, img = (int(x) for x in groups[g][:8])
            mem = [int(m) for m in groups[g][8:8 + n]]
            assert 1 <= n <= min(8, 128 // a)
            assert nch == -(-bef * aft // kc_of(a))
            for m in mem:
                assert m in stage_tasks
                ab, ao, _, _, _, _, tb, ta, tf = (int(x) for x in hp[m])
                assert (ab, ao, tb, ta, tf) == (Abuf, Aoff, bef, a, aft)
            seen += mem
            # items: ranges z = 0.. of the members' kchunk, covering every chunk once
            gi = sorted((int(z), int(c0), int(c1)) for gg, z, c0, c1 in its if int(gg) == g)
            splits, kchunk = int(hpx[mem[0]][0]), int(hpx[mem[0]][1])
            assert [z for z, _, _ in gi] == list(range(splits))
            assert kchunk % kc_of(a) == 0
            cpi = kchunk // kc_of(a)
            assert [(c0, c1) for _, c0, c1 in gi] == [(z * cpi, min(nch, (z + 1) * cpi)) for z in range(splits)]
            for m in mem:
                assert (int(hpx[m][0]), int(hpx[m][1])) == (splits, kchunk)
            key = (Abuf, Aoff, bef, a, aft)
            assert img_of.setdefault(key, img) == img  # one image per distinct A
        assert sorted(seen) == sorted(eligible)  # every qualifying task once
        # image units: every chunk of every distinct A exactly once, images disjoint
        owners = {}
        for g, c in units[htu0:htu0 + nhtu]:
            owners.setdefault(int(g), []).append(int(c))
        spans = []
        for g, cs in owners.items():
            nch, img, a = int(groups[g][6]), int(groups[g][7]), int(groups[g][3])
            assert sorted(cs) == list(range(nch))
            spans.append((img, img + nch * chunk_bytes(a, kc_of(a) // 16)))
        assert len(spans) == len(img_of)
        spans.sort()
        assert all(e0 <= s1 for (_, e0), (s1, _) in zip(spans, spans[1:]))
        assert all(0 <= s and e <= oz_bytes for s, e in spans)
        # workspace slots of split tasks (tensor-core and classic) disjoint
        ws = sorted((int(hpx[t][2]), int(hpx[t][2]) + int(hpx[t][0]) * int(hp[t][7]) ** 2)
                    for t in stage_tasks if int(hpx[t][0]) > 1)
        assert all(e0 <= s1 for (_, e0), (s1, _) in zip(ws, ws[1:]))
        assert all(e <= hpw for _, e in ws)
        # classic tiles: none for the tensor-core tasks
        assert not eligible & {int(t) for t, _, _ in tiles if t0 <= int(t) < t0 + nt}
        n_tc += len(eligible)
    if name in ("cfg4", "cfg1"):
        assert n_tc > 0


@pytest.mark.parametrize("flavour,prec", [(2, 1), (2 | TENSOR, 2)])
def test_no_tensor_core_hole_products_outside_double_float_tensor_plans(flavour, prec):
    tree, sop, _ = config_problem(4)
    pv = PlanView(tree, sop, flavour=flavour, prec=prec)
    assert len(pv.tables[52]) == 0 and len(pv.tables[53]) == 0


@pytest.mark.parametrize("name", ["cfg0", "cfg4", "cfg1", "wide_leaves"])
@pytest.mark.parametrize("plan", [1, 2])
def test_accumulation_items(name, plan):
    tree, sop = problem(name)
    pv = PlanView(tree, sop, flavour=plan | TENSOR, prec=1)
    T = pv.tables
    acc, tiles, items, units, ranges, imgs = T[3], T[49], T[57], T[58], T[59], T[60]
    oz_bytes = int(T[56][0])
    n_tc = 0
    for si, (kind, t0, nt, tile0, ntile) in enumerate(T[0]):
        ati0, nati, atu0, natu, nunits = (int(x) for x in ranges[si])
        if kind != ST_ACC:
            assert nati == 0 and natu == 0
            continue
        eligible = {t for t in range(t0, t0 + nt)
                    if int(acc[t][7]) >= 1 and acc_tc_eligible(int(acc[t][4]), int(acc[t][5]))}
        its = items[ati0:ati0 + nati]
        # items: every 128-row block of every eligible task once, units-before ascending
        blocks = {}
        pre = 0
        for task, blk, before, _ in its:
            assert int(before) == pre
            pre += int(acc[task][7])
            blocks.setdefault(int(task), []).append(int(blk))
        assert pre == nunits
        assert set(blocks) == eligible
        for t, b in blocks.items():
            assert sorted(b) == list(range(-(-int(acc[t][4]) // 128)))
        # image units: every term of every eligible task once; slots disjoint in B_OZ
        seen = sorted((int(t), int(s)) for t, s in units[atu0:atu0 + natu])
        assert seen == sorted((t, s) for t in eligible for s in range(int(acc[t][7])))
        spans = sorted((int(imgs[t]), int(imgs[t]) + int(acc[t][7]) * chunk_bytes(int(acc[t][5]), 4)) for t in eligible)
        assert all(e0 <= s1 for (_, e0), (s1, _) in zip(spans, spans[1:]))
        assert all(0 <= s and e <= oz_bytes for s, e in spans)
        for t in range(t0, t0 + nt):
            assert (int(imgs[t]) >= 0) == (t in eligible)
        # classic tiles: only the other tasks
        assert not eligible & {int(r[0]) for r in tiles[tile0:tile0 + ntile]}
        n_tc += len(eligible)
    if name in ("cfg4", "cfg1"):
        assert n_tc > 0
