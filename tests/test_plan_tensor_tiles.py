"""Planner side of the tensor-core mode products (flavour bit 0x8000 with
double-float or complex64 arithmetic), on the CPU: in every mode-product
stage the tasks with 32 <= a_in, a_out <= 64 (not diagonal) get tensor-core tiles
covering their rows exactly once and a slot of their own in the stage for
the operand image of h; every other task keeps its classic tiles, which
cover its output slots exactly once.  Image slots are private within a
stage and reused across stages (every stage's pre-pass rewrites them)."""
import numpy as np
import pytest

from plan_emulator import ST_MP, PlanView
from qutree_gb300.model import balanced_tree, config_problem, coupled_oscillators

TENSOR = 0x8000
OZ_ROWS = 16 * 8  # rows of one tensor-core tile (sub-tiles x rows per sub-tile)
MP_TILE = 256     # slots of one classic tile (b, four consecutive j, c)


def wide_leaf_problem():
    tree = balanced_tree(4, 80, 12)  # leaf operators 80 x 80: classic tiles
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=np.random.default_rng(8),
                              omega=1.0)
    return tree, sop


@pytest.mark.parametrize("problem", ["cfg0", "cfg4", "wide_leaves"])
@pytest.mark.parametrize("plan", [0, 1, 2])
def test_tensor_core_tiles_cover_eligible_tasks(problem, plan):
    if problem == "wide_leaves":
        tree, sop = wide_leaf_problem()
    else:
        tree, sop, _ = config_problem(int(problem[3:]))
    pv = PlanView(tree, sop, flavour=plan | TENSOR, prec=1)
    T = pv.tables
    mp, oz_tiles, ranges, oz_tasks, tiles = T[1], T[40], T[41], T[42], T[43]
    assert len(ranges) == len(T[0])
    for si, (kind, t0, nt, tile0, ntile) in enumerate(T[0]):
        oz0, noz, ozt0, nozt = ranges[si]
        slots = {}
        if kind != ST_MP:
            assert noz == 0 and nozt == 0
            continue
        eligible = {t for t in range(t0, t0 + nt)
                    if not mp[t][10] and 32 <= mp[t][7] <= 64 and 32 <= mp[t][8] <= 64}
        # tensor-core tiles: each eligible task's rows exactly once
        got = {}
        for task, q in oz_tiles[oz0:oz0 + noz]:
            got.setdefault(int(task), []).append(int(q))
        assert set(got) == eligible
        for t, qs in got.items():
            rows = int(mp[t][6]) * int(mp[t][9])
            assert sorted(qs) == list(range(-(-rows // OZ_ROWS)))
        # digits of h: one private slot per eligible task
        tasks = [int(t) for t, _ in oz_tasks[ozt0:ozt0 + nozt]]
        assert sorted(tasks) == sorted(eligible)
        for t, off in oz_tasks[ozt0:ozt0 + nozt]:
            assert off % 16 == 0
            slots[int(t)] = int(off)
        # classic tiles: the other tasks' outputs exactly once
        cl = {}
        for task, e0 in tiles[tile0:tile0 + ntile]:
            cl.setdefault(int(task), []).append(int(e0))
        assert set(cl) == set(range(t0, t0 + nt)) - eligible
        for t, starts in cl.items():
            n_slots = int(mp[t][6]) * (-(-int(mp[t][8]) // 4)) * int(mp[t][9])
            assert sorted(starts) == list(range(0, n_slots, MP_TILE))
        # slots disjoint: double-float plans hold the image of alpha h of the
        # sum-of-products kernel (4 steps x 7 digits x 3 ap rows x 16 bf16,
        # exponents), ap = a_out rounded up to 8
        spans = sorted((off, off + 4 * 7 * 3 * ((int(mp[t][8]) + 7) // 8 * 8) * 32 + 256) for t, off in slots.items())
        assert len(spans) == len(eligible)
        assert all(e0 <= s1 for (_, e0), (s1, _) in zip(spans, spans[1:]))
    if problem == "wide_leaves":  # the 80 x 80 leaf products keep classic tiles
        assert sum(int(n) for kind, _, _, _, n in T[0] if kind == ST_MP) > 0


def test_tensor_core_bit_needs_double_float():
    tree, sop, _ = config_problem(0)
    with pytest.raises(ValueError, match="double-float"):
        PlanView(tree, sop, flavour=2 | TENSOR, prec=0)


def test_plain_double_float_plan_has_no_tensor_core_tiles():
    tree, sop, _ = config_problem(0)
    pv = PlanView(tree, sop, flavour=2, prec=1)
    assert len(pv.tables[40]) == 0 and len(pv.tables[42]) == 0
