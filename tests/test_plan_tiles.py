"""Planner tiles of the tiled stages, on the CPU: in every stage of every
plan (sweep, frozen-matrix and SCF stages) the blocks of the mode products
(slots of four outputs), accumulations (64 rows x 16 columns), small matrix
products (256 outputs) and conversions (2048 elements) belong to the stage's
tasks and cover each task exactly once."""
import numpy as np
import pytest

from plan_emulator import ST_ACC, ST_CVT, ST_MM, ST_MP, PlanView
from qutree_gb300 import qtgpu
from qutree_gb300.model import balanced_tree, config_problem, coupled_oscillators


def problems():
    out = []
    for cfg in (0, 4):
        tree, sop, _ = config_problem(cfg)
        out.append((f"cfg{cfg}", tree, sop))
    tree = balanced_tree(7, 5, 4)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=np.random.default_rng(2),
                              omega=1.0)
    out.append(("tree7", tree, sop))
    return out


PROBLEMS = problems()


def expected(kind, row):
    """Tile starts of one task."""
    if kind == ST_MP:
        before, a_out, after = int(row[6]), int(row[8]), int(row[9])
        return [(s,) for s in range(0, before * -(-a_out // 4) * after, 256)]
    if kind == ST_ACC:
        rows, d = int(row[4]), int(row[5])
        return [(r, j) for r in range(0, rows, 64) for j in range(0, d, 16)]
    if kind == ST_MM:
        d = int(row[2])
        return [(e,) for e in range(0, d * d, 256)]
    n = int(row[4])  # ST_CVT
    return [(e,) for e in range(0, n, 2048)]


@pytest.mark.parametrize("flavour", [0, 1, 2, 2 | qtgpu.QT_PLAN_SCF])
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("name,tree,sop", PROBLEMS, ids=[p[0] for p in PROBLEMS])
def test_tiles_cover_every_task_once(name, tree, sop, prec, flavour):
    if flavour & qtgpu.QT_PLAN_SCF and flavour & 0xFF != 2:
        pytest.skip("the SCF sweep needs the compressed plan")
    pv = PlanView(tree, sop, flavour=flavour, prec=prec)
    T = pv.tables
    table = {ST_MP: (1, 43), ST_ACC: (3, 49), ST_MM: (22, 50), ST_CVT: (18, 51)}
    checked = set()
    for kind, t0, nt, tile0, ntile in T[0]:
        if kind not in table:
            continue
        tasks, tiles = T[table[kind][0]], T[table[kind][1]]
        got = {}
        for tl in tiles[tile0:tile0 + ntile]:
            t = int(tl[0])
            assert t0 <= t < t0 + nt
            got.setdefault(t, []).append(tuple(int(x) for x in tl[1:]))
        for t in range(t0, t0 + nt):
            want = expected(kind, tasks[t])
            assert sorted(got.get(t, [])) == sorted(want)
        checked.add(int(kind))
    assert ST_MP in checked and ST_ACC in checked
