"""Generate tests/golden/oracle_cases.npz: outputs of the oracle (the C
restatement of the FastS solve step) on small seeded cases of every scheme
family of the path.

The reference itself cannot run here (Fortran sources, Cassiopee absent),
so these vectors pin the oracle against unintended change and give the GPU
tests a fixed target.  Per case: 512 values of the final state at seeded
positions (ghosts included), the interior sum of each variable, and (for
implicit cases) the Newton residual norms of the last step.  The case
inputs are rounded to a coarse binary grid first (see quantized), so the
vectors are platform independent.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT), str(ROOT / "oracle")]

from fast_gb300 import cases, fasts  # noqa: E402

NSAMPLE = 512


def specs():
    """name -> (builder, steps, nstep_fin, modulo_verif).  The builders are
    small seeded / deterministic cases (cases.py)."""
    return {
        "vortex_roe_minmod_rk3": (
            lambda: cases.isentropic_vortex(n=(24, 20, 6), numz={"scheme": "roe_min", "slope": "minmod",
                                                                 "time_step": 0.05}), 3, 3, 1000),
        "vortex_roe_o3_wavy_rk3": (
            lambda: cases.isentropic_vortex(n=(20, 16, 6), wavy=0.3,
                                            numz={"scheme": "roe", "slope": "o3", "time_step": 0.05}),
            3, 3, 1000),
        "tgv_ausm_lusgs": (
            lambda: cases.taylor_green(n=(12, 10, 8), ss_iteration=3), 2, 4, 1),
        "tgv_senseur_wavy_visc_rk3": (
            lambda: cases.taylor_green(n=(12, 10, 8), wavy=0.3, reynolds=200.0, scheme="senseur",
                                       slope="o3", dt=0.02,
                                       numb={"temporal_scheme": "explicit", "ss_iteration": 1,
                                             "modulo_verif": 1000}), 3, 3, 1000),
        "bcbox_wavy_ns_lusgs": (
            lambda: cases.bc_box(n=(12, 10, 6), wall="BCWallViscous", model="NSLaminar", wavy=0.3,
                                 temporal="implicit", ss_iteration=3, time_step=0.05,
                                 reynolds=500.0), 2, 4, 1),
        "bcbox_sa_rk3": (
            lambda: cases.bc_box(n=(12, 10, 6), wall="BCWallViscous", model="NSTurbulent",
                                 temporal="explicit", time_step=0.02, reynolds=500.0), 3, 3, 1000),
        "bcbox_sa_wavy_lusgs": (
            lambda: cases.bc_box(n=(12, 10, 6), wall="BCWallViscous", model="NSTurbulent", wavy=0.3,
                                 temporal="implicit", ss_iteration=3, time_step=0.05,
                                 reynolds=500.0), 2, 4, 1),
    }


QUANTUM = 2.0 ** -20


def quantized(t, coords):
    """The case with its initial conservative fields (and, for curvilinear
    meshes, its coordinates) rounded to multiples of QUANTUM: numpy's sin /
    exp may differ in the last bit between host architectures, and rounding
    makes the inputs identical everywhere (a 1-ulp difference straddles a
    rounding boundary with probability ~ulp/QUANTUM ~ 2^-32 per value)."""
    from fast_gb300 import pytree as I
    z = I.getZones(t)[0]
    sol = I.getNodeFromName1(z, I.__FlowSolutionCenters__)
    for node in sol[2]:
        if isinstance(node[1], np.ndarray) and node[1].dtype == np.float64:
            node[1] = np.asfortranarray(np.round(node[1] / QUANTUM) * QUANTUM)
    if coords:
        gc = I.getNodeFromName1(z, "GridCoordinates")
        for node in gc[2]:
            node[1] = np.asfortranarray(np.round(node[1] / QUANTUM) * QUANTUM)
    return t


def build_case(name):
    """The quantized tree of case `name` and its run parameters."""
    build, steps, nstep_fin, mv = specs()[name]
    return quantized(build(), "wavy" in name), steps, nstep_fin, mv


def positions(size, seed):
    return np.sort(np.random.default_rng(seed).choice(size, NSAMPLE, replace=False))


def interior_sums(pi, q):
    ni, nj, nk = (int(pi[0]), int(pi[1]), int(pi[2]))
    ng, ngk = int(pi[3]), int(pi[4])
    a = q.reshape(int(pi[36]), nk, nj, ni)[:, ngk:nk - ngk, ng:nj - ng, ng:ni - ng]
    return a.sum(axis=(1, 2, 3))


def run_oracle(name):
    import oracle
    t, steps, nstep_fin, mv = build_case(name)
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle.Case(zd)
    c.apply_bc(0)
    c.apply_bc(1)
    for it in range(1, steps + 1):
        c.compute(it, 1, nstep_fin, 1, modulo_verif=mv)
    q = c.z[0]["lv"][0]
    pi = zd[0]["pi"]
    norms = c.residual_norms(0, int(pi[58])) if mv == 1 else np.zeros((0,))
    return zd, q, norms


def main():
    import oracle
    oracle.build()
    out = {}
    for i, name in enumerate(specs()):
        zd, q, norms = run_oracle(name)
        pos = positions(q.size, 1000 + i)
        out[name + "/pos"] = pos
        out[name + "/val"] = q[pos]
        out[name + "/sum"] = interior_sums(zd[0]["pi"], q)
        out[name + "/norms"] = np.asarray(norms)
        print(name, q.size, out[name + "/sum"])
    np.savez_compressed(Path(__file__).with_name("oracle_cases.npz"), **out)


if __name__ == "__main__":
    main()
