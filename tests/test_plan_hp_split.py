"""Planner side of the hole products split over their reduction index, on
the CPU: in every hole-product stage each task's output tiles times its
reduction ranges are covered by exactly one block; the ranges span the
reduction index (at least 64 rows each, multiples of 16, unless the whole
index is shorter); split tasks own disjoint workspace slots inside the
workspace; the stage's launches cover its tiles, one register-tile shape
each; and the partial tiles are summed exactly when a task is split."""
import numpy as np
import pytest

from plan_emulator import ST_HP, PlanView
from qutree_gb300.model import balanced_tree, config_problem, coupled_oscillators

TILE = 64


def problems():
    out = []
    for cfg in (0, 4):
        tree, sop, _ = config_problem(cfg)
        out.append((f"cfg{cfg}", tree, sop))
    for leaves, p, b in ((7, 5, 4), (16, 16, 12), (4, 80, 12)):
        tree = balanced_tree(leaves, p, b)
        sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=np.random.default_rng(3),
                                  omega=1.0)
        out.append((f"tree{leaves}_{p}_{b}", tree, sop))
    return out


PROBLEMS = problems()


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("plan", [0, 1, 2])
@pytest.mark.parametrize("name,tree,sop", PROBLEMS, ids=[p[0] for p in PROBLEMS])
def test_hole_product_blocks_cover_every_task_once(name, tree, sop, plan, prec):
    pv = PlanView(tree, sop, flavour=plan, prec=prec)
    T = pv.tables
    hp, split, tiles, segs, ranges = T[2], T[44], T[45], T[46], T[47]
    wsize = int(T[48][0])
    assert len(split) == len(hp) and len(ranges) == len(T[0])
    for si, (kind, t0, nt, tile0, ntile) in enumerate(T[0]):
        if kind != ST_HP:
            continue
        seg0, nseg, aux = ranges[si]
        # launches: contiguous, covering the stage's tiles, one shape each
        pos = tile0
        for rows, cols, first, count in segs[seg0:seg0 + nseg]:
            assert first == pos and count > 0
            for t, _, _ in tiles[first:first + count]:
                assert (split[t][3], split[t][4]) == (rows, cols)
            pos += count
        assert pos == tile0 + ntile
        # every (output tile, reduction range) of every task exactly once
        seen = {}
        for t, y, z in tiles[tile0:tile0 + ntile]:
            assert t0 <= t < t0 + nt
            seen.setdefault(int(t), []).append((int(y), int(z)))
        assert set(seen) == set(range(t0, t0 + nt))
        slots = []
        for t in range(t0, t0 + nt):
            a, K = int(hp[t][7]), int(hp[t][6]) * int(hp[t][8])
            splits, kchunk, ws = int(split[t][0]), int(split[t][1]), int(split[t][2])
            nti = -(-a // TILE)
            assert sorted(seen[t]) == [(y, z) for y in range(nti * nti) for z in range(splits)]
            # the ranges span the reduction index
            assert (splits - 1) * kchunk < K <= splits * kchunk
            if kchunk < K:
                assert kchunk >= 64 and kchunk % 16 == 0
            if splits > 1:
                slots.append((ws, ws + splits * a * a))
        # split tasks: disjoint workspace slots inside the workspace; summed iff any
        slots.sort()
        assert all(e <= s for (_, e), (s, _) in zip(slots, slots[1:]))
        assert all(0 <= s and e <= wsize for s, e in slots)
        assert bool(aux) == bool(slots)
