"""The oracle over every tree of a batched forest, spread over host
processes.  Each worker rebuilds the (seeded, deterministic) forest and runs
the oracle's BLAS-backed sweep on a contiguous slice of its trees; nothing
here touches CUDA, and the pool is started with the spawn method, so it is
safe after the parent has used the GPU."""
import multiprocessing as mp
import os

import numpy as np


def _slice(args):
    n_trees, k0, k1 = args
    import oracle as O
    from qutree_gb300.model import batched_problem
    O.attach_openblas(fast=True)
    trees, sops, psis = batched_problem(n_trees)
    out = []
    for k in range(k0, k1):
        r = O.derivative(trees[k], sops[k], psis[k].flat(), backend=O.BLAS, fast=True)
        out.append((k, float(r.energy), np.asarray(r.dpsi), np.asarray(r.rho)))
    return out


def oracle_forest(n_trees, workers=None):
    """[(energy, dpsi, rho)] of every tree of batched_problem(n_trees)."""
    workers = workers or max(1, min(16, os.cpu_count() or 1))
    step = -(-n_trees // workers)
    jobs = [(n_trees, k, min(n_trees, k + step)) for k in range(0, n_trees, step)]
    env = {"OPENBLAS_NUM_THREADS": "1", "OMP_NUM_THREADS": "1"}
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        with mp.get_context("spawn").Pool(len(jobs)) as pool:
            parts = pool.map(_slice, jobs)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    res = [None] * n_trees
    for part in parts:
        for k, e, d, r in part:
            res[k] = (e, d, r)
    return res
