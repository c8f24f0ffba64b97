"""Generate the golden fixtures of the LLG path by running the reference (magex) itself.

Run in a container where the reference source tree is available (read-only is fine):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/magex

It imports magex from that tree and writes, next to this file:
  models.json      magex make_model dicts and the load_results coupling lists of a set of models
  llg_golden.npz   LLGSolver trajectories (NumPy Heun / Depondt path, the reference's own stream of
                   thermal noise), observables, run() tables and topological charges

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/magex --thermal-bcc2

writes only thermal_bcc2.npz: the equilibrium statistics of magex's own Langevin run of the
benchmark Hamiltonian (two-site bcc, full 3x3 tensors with DMI, SIA, B_z = 0.5 T, 300 K) at 8^3
cells (eight runs in parallel processes, about 5 minutes on 8 cores);  --adversarial writes only adversarial.npz: T = 0
trajectories of models whose couplings span eight decades in one stencil, in a 100 T field.

The fixtures are inputs and outputs of the reference, not data of any public benchmark; every model
is a seeded synthetic lattice.  numpy / scipy versions are recorded in the npz.
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))      # the repo, for the bcc model generator


def main(ref_root):
    sys.path.insert(0, ref_root)
    import scipy
    from magex import models as RM
    from magex import spinmodel as RS
    from magex import texture as RT
    from magex.llg import LLGSolver
    from magex.structure import apply_structure
    from magex_gb300.workloads import bcc_two_site_model

    tmp = tempfile.mkdtemp()
    out = {"numpy_version": np.array(np.__version__), "scipy_version": np.array(scipy.__version__)}
    models = {}

    def uc_of(name, d):
        p = os.path.join(tmp, name + ".json")
        with open(p, "w") as f:
            json.dump(d, f)
        uc = RS.load_results(p)
        models[name] = dict(
            model=d,
            couplings=[[int(i), int(j), [int(x) for x in R], np.asarray(J).tolist()] for i, j, R, J in uc.couplings],
            A=np.asarray(uc.A).tolist(), moments=np.asarray(uc.moments).tolist(),
            signs=np.asarray(uc.signs).tolist(),
            info={k: uc.info[k] for k in ("rcut", "nn_distance", "shells", "ncouplings_per_cell", "J0_fraction")})
        return uc

    # ---------------------------------------------------------------- models (make_model kwargs)
    kw_cases = {
        "sc": dict(lattice="sc", a=3.0, J=[1.0], moment=2.0),
        "sc_dmi": dict(lattice="sc", J=[1.0], D=0.1, K=0.05),
        "sc_two_shell": dict(lattice="sc", J=[1.0, 0.3], D=0.1, K=0.05),
        "sc_afm": dict(lattice="sc", J=[-1.0], order="afm"),
        "sc_open": dict(lattice="sc", J=[1.0], D=0.2, K=0.1),
        "tri": dict(lattice="triangular", a=3.0, J=[1.0], D=0.3, dmi="interfacial", K=0.05, moment=2.0),
        "tri_two_shell": dict(lattice="triangular", J=[1.0, 0.2], D=0.3, K=0.1),
        "honeycomb_bulk": dict(lattice="honeycomb", J=[1.0, 0.1, 0.05], D=0.2, dmi="bulk"),
        "bcc1": dict(lattice="bcc", J=[1.0, 0.3]),
        "fcc_jani": dict(lattice="fcc", J=[1.0], Jani=[[0.01, 0, 0], [0, 0.02, 0], [0, 0, -0.03]]),
        "kagome": dict(lattice="kagome", J=[1.0], D=0.1),
    }
    ucs = {}
    for name, kw in kw_cases.items():
        models[name + "__kwargs"] = kw
        ucs[name] = uc_of(name, RM.make_model(**kw))
    ucs["bcc2"] = uc_of("bcc2", bcc_two_site_model(J=(20.0, 10.0, -1.0), seed=0))
    ucs["bcc2_shell4"] = uc_of("bcc2_shell4", bcc_two_site_model(J=(20.0, 10.0, -1.0, 1.0), dmi_frac=0.05,
                                                                 per="shell", seed=1))

    # ---------------------------------------------------------------- trajectories
    def traj(tag, uc, L, pbc, B, alpha, dt, T, seed, steps, keep, integrator="heun", init_seed=None,
             structure=None, run_every=None):
        s = RS.SpinSystem(uc, L, pbc, B)
        if structure:
            apply_structure(s, structure)
        e = s.init_spins("random", seed=seed if init_seed is None else init_seed)
        sol = LLGSolver(s, alpha, dt, T, seed, integrator=integrator)
        out[f"{tag}/e0"] = e.copy()
        for n in range(1, steps + 1):
            e = sol.step(e)
            if n in keep:
                out[f"{tag}/e{n}"] = e.copy()
        out[f"{tag}/energy"] = np.array(s.energy(e))
        out[f"{tag}/order"] = np.array(s.order_parameter(e))
        out[f"{tag}/torque"] = np.array(sol.max_torque(e))
        out[f"{tag}/field"] = s.effective_field(e)
        if run_every:
            s2 = RS.SpinSystem(uc, L, pbc, B)
            if structure:
                apply_structure(s2, structure)
            sol2 = LLGSolver(s2, alpha, dt, T, seed, integrator=integrator)
            _, tab, _ = sol2.run(out[f"{tag}/e0"].copy(), steps, output_every=run_every)
            out[f"{tag}/table"] = tab
        meta = dict(L=list(L), pbc=[bool(x) for x in pbc], B=list(map(float, B)), alpha=alpha, dt=dt, T=T, seed=seed,
                    steps=steps, keep=sorted(keep), integrator=integrator, structure=structure, run_every=run_every,
                    init_seed=seed if init_seed is None else init_seed)
        models["traj__" + tag] = meta

    # config-1 workload: sc 16^3, J = 1 meV, mu = 2, alpha 0.1, dt 0.1 fs, T = 0, 1000 steps
    traj("sc16", ucs["sc"], (16, 16, 16), (1, 1, 1), (0, 0, 0), 0.1, 1e-4, 0.0, 1, 1000, {1, 10, 100, 1000},
         run_every=100)
    # thermal, the reference's own noise stream (default_rng(seed).normal per step)
    traj("sc6_thermal", ucs["sc_dmi"], (6, 6, 6), (1, 1, 1), (0.1, 0, 0.5), 0.2, 1e-3, 50.0, 5, 20, {1, 5, 20},
         run_every=5)
    # config-2 Hamiltonian on a 4^3 copy: full tensors, DMI, SIA, Zeeman, T = 300 K
    traj("bcc2_thermal", ucs["bcc2"], (4, 4, 4), (1, 1, 1), (0, 0, 0.5), 0.05, 1e-4, 300.0, 7, 20, {1, 20})
    traj("bcc2_T0", ucs["bcc2"], (4, 4, 4), (1, 1, 1), (0, 0, 0.5), 0.05, 1e-4, 0.0, 8, 100, {1, 100},
         run_every=25)
    traj("bcc2_shell4", ucs["bcc2_shell4"], (4, 4, 4), (1, 1, 1), (0, 0, 0.2), 0.05, 1e-4, 600.0, 9, 10, {10})
    # config-4 Hamiltonian on a 16x16 copy (T = 0, alpha 0.3, B_z = 2 T)
    traj("tri16", ucs["tri"], (16, 16, 1), (1, 1, 0), (0, 0, 2.0), 0.3, 1e-4, 0.0, 4, 200, {1, 200}, run_every=50)
    # Depondt (magex tests/cuda_sim_check.py model), T = 0 and T > 0
    traj("sc_depondt", ucs["sc_dmi"], (4, 4, 3), (1, 1, 1), (0.1, 0, 0.5), 0.2, 1e-3, 0.0, 1, 20, {1, 20},
         integrator="depondt")
    traj("tri_depondt_thermal", ucs["tri"], (8, 8, 1), (1, 1, 0), (0, 0, 2.0), 0.3, 1e-3, 10.0, 2, 20, {20},
         integrator="depondt")
    # edge cases: open boundaries, self-image folding and repeated neighbours, AFM two-sublattice cell
    traj("sc_open", ucs["sc_open"], (5, 5, 4), (0, 0, 0), (0.2, 0, 2.0), 0.1, 1e-3, 0.0, 2, 20, {20})
    traj("sc_tiny_fold", ucs["sc_two_shell"], (1, 2, 3), (1, 1, 1), (0, 0, 0.3), 0.1, 1e-3, 5.0, 2, 20, {20})
    traj("sc_afm", ucs["sc_afm"], (3, 3, 3), (1, 1, 1), (0, 0, 0), 0.5, 2e-3, 0.0, 2, 50, {50}, run_every=10)
    traj("honeycomb", ucs["honeycomb_bulk"], (6, 5, 1), (1, 1, 0), (0, 0.1, 0.3), 0.1, 1e-3, 3.0, 3, 10, {10})
    # structure: per-material damping and temperature, pinned bottom layer, site temperature profile
    st = dict(materials=[dict(name="bulk", alpha=0.3, T=40.0)], pinned=[dict(region="bottom", layers=1,
                                                                                  direction=[0, 0, 1])],
              temperature_profile=dict(axis="x", T0=5.0, T1=30.0))
    traj("sc_structure", ucs["sc_dmi"], (6, 6, 4), (1, 1, 1), (0, 0, 0.5), 0.1, 1e-3, 10.0, 6, 10, {10},
         structure=st)
    # cubic and higher uniaxial anisotropy (magex/terms.py:35-75, added by magex/structure.py:163-193)
    c30, s30 = float(np.cos(np.pi / 6)), float(np.sin(np.pi / 6))
    traj("sc_cubic", ucs["sc_dmi"], (5, 5, 4), (1, 1, 1), (0.1, 0, 0.3), 0.1, 1e-3, 0.0, 3, 20, {1, 20},
         structure=dict(materials=[dict(name="bulk", Kc=0.3, K2=0.2, K3=0.1, K_axis=[1, 1, 1])]), run_every=5)
    traj("tri_cubic_thermal", ucs["tri"], (6, 6, 1), (1, 1, 0), (0, 0, 0.5), 0.2, 1e-3, 5.0, 4, 20, {20},
         integrator="depondt", structure=dict(materials=[dict(
             name="bulk", Kc=-0.2, cubic_axes=[[c30, -s30, 0.0], [s30, c30, 0.0], [0.0, 0.0, 1.0]], K2=0.1)]))
    # arbitrary lattices (per-site neighbour lists): a carved sphere with vacancies, and two materials
    # with interface exchange scaling; the reference's coupling matrix and per-site arrays are stored
    def irregular(tag, uc, L, pbc, B, structure, alpha, dt, T, seed, steps):
        s = RS.SpinSystem(uc, L, pbc, B)
        apply_structure(s, structure)
        J = s.Jsp.tocsr()
        out[f"{tag}/Jsp_indptr"] = J.indptr.astype(np.int64)
        out[f"{tag}/Jsp_indices"] = J.indices.astype(np.int64)
        out[f"{tag}/Jsp_data"] = J.data
        out[f"{tag}/A"] = np.asarray(s.A, float)
        out[f"{tag}/mu"] = np.asarray(s.mu, float)
        out[f"{tag}/signs"] = np.asarray(s.signs, float)
        for name in ("pinned", "site_T", "alpha_site"):
            v = getattr(s, name, None)
            if v is not None:
                out[f"{tag}/{name}"] = np.asarray(v)
        e = s.init_spins("random", seed=seed)
        sol = LLGSolver(s, alpha, dt, T, seed)
        out[f"{tag}/e0"] = e.copy()
        for _ in range(steps):
            e = sol.step(e)
        out[f"{tag}/e{steps}"] = e.copy()
        out[f"{tag}/energy"] = np.array(s.energy(e))
        out[f"{tag}/torque"] = np.array(sol.max_torque(e))
        models["irregular__" + tag] = dict(L=list(L), pbc=[bool(x) for x in pbc], B=list(map(float, B)),
                                           alpha=alpha, dt=dt, T=T, seed=seed, steps=steps, N=int(s.N))

    irregular("sc_sphere", ucs["sc_dmi"], (9, 9, 9), (0, 0, 0), (0.1, 0.0, 0.4),
              dict(shape="sphere", size=11.0, vacancies=dict(fraction=0.1, seed=3)), 0.2, 1e-3, 20.0, 4, 20)
    irregular("sc_interface", ucs["sc_dmi"], (6, 6, 6), (1, 1, 1), (0.0, 0.0, 0.5),
              dict(layers=[dict(material="A", thickness=3), dict(material="B", thickness=3)],
                   exchange_scale=[[1.0, 0.5], [0.5, 0.8]],
                   pinned=[dict(region="bottom", layers=1)]), 0.1, 1e-3, 0.0, 5, 20)

    # time-dependent uniform field (field_func) and state-dependent per-site field (extra_field) on the
    # solver, magex/llg.py:124-137; the callables are rebuilt from these parameters by the tests
    sys.path.insert(0, os.path.dirname(HERE))
    from helpers import callable_fields, site_field_func
    cparams = dict(pulse=[0.05, 0.0, 0.0], t0=4.5 * 2e-3, amp=0.1, w=50.0, k=[0.0, 0.0, 1.0], c=0.2)
    sot = dict(p=[0.3, 1.0, 0.2], B_DL=0.4, B_FL=0.15)
    ff, xf = callable_fields(cparams)
    models["callables"] = dict(params=cparams, sot=sot, cases={})
    # use_ff: 0 none, 1 uniform field_func, 2 per-site field_func
    for tag, model, L, pbc, B, alpha, dt, steps, keep, use_ff, use_xf, use_sot, integ in (
            ("pulse", "sc_dmi", (5, 5, 2), (1, 1, 1), (0.0, 0.0, 0.3), 0.02, 2e-3, 30, {4, 5, 30}, 1, False, False,
             "heun"),
            ("extra", "sc_dmi", (4, 4, 4), (1, 1, 1), (0.1, 0.0, 0.4), 0.1, 1e-3, 20, {1, 20}, 0, True, False, "heun"),
            ("both", "tri", (6, 6, 1), (1, 1, 0), (0.0, 0.0, 1.0), 0.05, 1e-3, 15, {1, 15}, 1, True, False, "depondt"),
            ("sot", "sc_dmi", (4, 4, 4), (1, 1, 1), (0.0, 0.0, 0.2), 0.05, 1e-3, 20, {1, 20}, 0, False, True, "heun"),
            ("sot_site", "tri", (6, 6, 1), (1, 1, 0), (0.0, 0.0, 1.0), 0.05, 1e-3, 15, {1, 15}, 2, False, True,
             "depondt")):
        s = RS.SpinSystem(ucs[model], L, pbc, B)
        sol = LLGSolver(s, alpha, dt, 0.0, 3, integrator=integ, sot=sot if use_sot else None)
        sol.field_func = {0: None, 1: ff, 2: site_field_func(cparams, s.N)}[use_ff]
        sol.extra_field = xf if use_xf else None
        e = s.init_spins("random", seed=4)
        out[f"callables/{tag}/e0"] = e.copy()
        out[f"callables/{tag}/field0"] = sol.field(e, 0.0)
        out[f"callables/{tag}/rhs0"] = sol.rhs(e, 0.0, 0.0)
        for n in range(1, steps + 1):
            e = sol.step(e)
            if n in keep:
                out[f"callables/{tag}/e{n}"] = e.copy()
        out[f"callables/{tag}/torque"] = np.array(sol.max_torque(e))
        models["callables"]["cases"][tag] = dict(model=model, L=list(L), pbc=[bool(x) for x in pbc], B=list(B),
                                                  alpha=alpha, dt=dt, steps=steps, keep=sorted(keep),
                                                  field_func=use_ff, extra_field=use_xf, sot=use_sot,
                                                  integrator=integ)

    # run() loop semantics (magex/llg.py:254-283): early stop on torque_tol (T = 0), and a callback that
    # changes the temperature every step (the two-temperature hook of magex/llg.py:337-341) with snapshots
    s = RS.SpinSystem(ucs["sc_afm"], (3, 3, 3), (1, 1, 1), (0, 0, 0))
    e0 = s.init_spins("reference", cone=0.3, seed=2)
    sol = LLGSolver(s, 0.5, 2e-3, 0.0, 2)
    e, tab, _ = sol.run(e0.copy(), 4000, output_every=100, torque_tol=1e-3)
    out["run_tol/e0"], out["run_tol/e"], out["run_tol/table"] = e0, e, tab
    s = RS.SpinSystem(ucs["sc_dmi"], (4, 4, 4), (1, 1, 1), (0.0, 0.0, 0.5))
    e0 = s.init_spins("random", seed=6)
    sol = LLGSolver(s, 0.1, 1e-3, 20.0, 8)
    seen = []

    def cool(n, e_, solver=sol):
        seen.append([n, float(e_[0, 2])])
        solver.T = 20.0 * np.exp(-0.05 * n)
    e, tab, snaps = sol.run(e0.copy(), 40, output_every=10, snapshots=4, callback=cool)
    out["run_cb/e0"], out["run_cb/e"], out["run_cb/table"] = e0, e, tab
    out["run_cb/seen"] = np.array(seen)
    out["run_cb/snap_t"] = np.array([t for t, _ in snaps])
    out["run_cb/snap_last"] = snaps[-1][1]

    # one draw of LLGSolver.thermal_field (magex/llg.py:106-122) of the sc6_thermal system
    s = RS.SpinSystem(ucs["sc_dmi"], (6, 6, 6), (1, 1, 1), (0.1, 0, 0.5))
    out["thermal_field/b"] = LLGSolver(s, 0.2, 1e-3, 50.0, 5).thermal_field()

    # Larmor precession of one free spin (magex tests/test_spindyn.py:36-45)
    s = RS.SpinSystem(uc_of("free", RM.make_model("sc", J=[0.0])), (1, 1, 1), field=(0, 0, 2.0))
    sol = LLGSolver(s, alpha=0.0, dt=1e-3)
    e = np.array([[1.0, 0, 0]])
    ph = []
    for _ in range(1000):
        e = sol.step(e)
        ph.append(np.arctan2(e[0, 1], e[0, 0]))
    out["larmor/e1000"] = e
    out["larmor/phase"] = np.unwrap(np.array(ph))

    # ---------------------------------------------------------------- thermal equilibrium statistics
    # Langevin run of an sc ferromagnet below T_c with the reference's noise stream; block means of
    # E/N and |M| (20 blocks) give the means and their standard errors that a run with any other
    # noise stream must reproduce within 3 sigma.
    th = dict(L=8, alpha=0.5, dt=2e-3, T=15.0, Bz=0.2, seed=21, equil=3000, sample=40000, every=20)
    s = RS.SpinSystem(ucs["sc"], (th["L"],) * 3, (1, 1, 1), (0.0, 0.0, th["Bz"]))
    sol = LLGSolver(s, alpha=th["alpha"], dt=th["dt"], temperature=th["T"], seed=th["seed"])
    e = s.init_spins("ferro")
    for _ in range(th["equil"]):
        e = sol.step(e)
    Es, Ms = [], []
    for k in range(th["sample"]):
        e = sol.step(e)
        if k % th["every"] == th["every"] - 1:
            Es.append(s.energy(e, per_spin=True))
            Ms.append(np.linalg.norm(e.mean(0)))
    for key, x in (("E", np.array(Es)), ("M", np.array(Ms))):
        blocks = x.reshape(20, -1).mean(1)
        out[f"thermal/{key}_mean"] = np.array(blocks.mean())
        out[f"thermal/{key}_sem"] = np.array(blocks.std(ddof=1) / np.sqrt(20))
    out["thermal/params"] = np.array(json.dumps(th))

    # ---------------------------------------------------------------- Monte Carlo (magex/montecarlo.py)
    from magex import montecarlo as RMC

    def mc_traj(tag, uc, L, pbc, B, T, seed, move, overrelax, sigma, sweeps, init_seed, structure=None):
        s = RS.SpinSystem(uc, L, pbc, B)
        if structure:
            apply_structure(s, structure)
        mc = RMC.MetropolisMC(s, T, seed, sigma, overrelax, move)
        assert mc.fast is None, "the golden MC runs use magex's NumPy sweep"
        e = s.init_spins("random", seed=init_seed)
        out[f"mc/{tag}/e0"] = e.copy()
        out[f"mc/{tag}/colour"] = RMC.greedy_coloring(s.N, s.bonds).astype(np.int32)
        acc = []
        for k in range(1, sweeps + 1):
            e = mc.sweep(e)
            out[f"mc/{tag}/e{k}"] = e.copy()
            acc.append([mc.accepted, mc.tried])
        out[f"mc/{tag}/accepted_tried"] = np.array(acc, np.int64)
        out[f"mc/{tag}/energy"] = np.array(s.energy(e))
        models["mc__" + tag] = dict(model=None, L=list(L), pbc=[bool(x) for x in pbc], B=list(map(float, B)),
                                    T=T, seed=seed, move=move, overrelax=overrelax, sigma=sigma, sweeps=sweeps,
                                    structure=structure, N=int(s.N), ncolors=mc.ncolors)

    mc_traj("gauss_dmi", ucs["sc_dmi"], (6, 6, 6), (1, 1, 1), (0.1, 0.0, 0.4), 10.0, 3, "gaussian", 1, 0.6, 5, 1)
    mc_traj("uniform_sc", ucs["sc"], (4, 4, 4), (1, 1, 1), (0.0, 0.0, 0.0), 20.0, 4, "uniform", 0, 0.6, 5, 2)
    mc_traj("heatbath_tri", ucs["tri"], (8, 8, 1), (1, 1, 0), (0.0, 0.0, 1.0), 5.0, 5, "heatbath", 1, 0.6, 5, 3)
    mc_traj("hinzke_bcc2", ucs["bcc2"], (2, 2, 2), (1, 1, 1), (0.0, 0.0, 0.5), 300.0, 6, "hinzke", 0, 0.4, 5, 4)
    mc_traj("T0_afm", ucs["sc_afm"], (4, 4, 4), (1, 1, 1), (0.0, 0.0, 0.0), 0.0, 7, "heatbath", 1, 0.3, 5, 5)
    mc_traj("open_kagome", ucs["kagome"], (4, 3, 1), (0, 0, 0), (0.0, 0.2, 0.1), 8.0, 8, "gaussian", 2, 0.5, 4, 6)
    mc_traj("structure", ucs["sc_dmi"], (6, 6, 4), (1, 1, 1), (0, 0, 0.5), 10.0, 9, "heatbath", 1, 0.6, 4, 7,
            structure=st)
    mc_traj("bcc2_shell4", ucs["bcc2_shell4"], (3, 3, 3), (1, 1, 1), (0.0, 0.0, 0.2), 150.0, 10, "gaussian", 1,
            0.3, 3, 8)
    mc_traj("cubic", ucs["sc_dmi"], (4, 4, 4), (1, 1, 1), (0.0, 0.1, 0.3), 8.0, 12, "gaussian", 1, 0.6, 4, 10,
            structure=dict(materials=[dict(name="bulk", Kc=0.4, K2=0.3, K3=0.1, K_axis=[0, 1, 1])]))
    mc_traj("cubic_heatbath", ucs["sc_dmi"], (4, 4, 4), (1, 1, 1), (0.0, 0.1, 0.3), 8.0, 13, "heatbath", 1, 0.6, 4,
            11, structure=dict(materials=[dict(name="bulk", Kc=-0.3)]))
    # carved sphere with vacancies (neighbour lists): the structure of the sc_sphere LLG case
    mc_traj("sphere", ucs["sc_dmi"], (9, 9, 9), (0, 0, 0), (0.1, 0.0, 0.4), 6.0, 11, "gaussian", 1, 0.6, 3, 9,
            structure=dict(shape="sphere", size=11.0, vacancies=dict(fraction=0.1, seed=3)))

    # one (L, T) point of magex's Monte Carlo run (equilibrium E, C, m, chi, U4 with 10-block errors)
    cpt = dict(sigma=0.6, overrelax=1, move="gaussian", init="ferro", init_axis=(0, 0, 1), therm_sweeps=1000,
               meas_sweeps=4000, sample_every=2)
    row = RMC._point((ucs["sc"], (8, 8, 8), (1, 1, 1), (0.0, 0.0, 0.0), 25.0, cpt, 12))
    models["mc_point"] = dict(c=cpt, L=[8, 8, 8], T=25.0, seed=12,
                              row={k: (float(v) if np.isscalar(v) else v) for k, v in row.items()
                                   if k not in ("spins", "seconds", "mvec")})

    # parallel tempering (magex/advanced_mc.py:38-95): sc 6^3 replicas around T_c, the reference's rows
    # and swap acceptances (compared within statistical errors: the sweeps draw other random numbers)
    from magex.advanced_mc import parallel_tempering
    pt = dict(L=[6, 6, 6], T=[32.0, 34.0, 36.0, 38.0, 40.0], therm=1000, meas=4000, sample_every=2, swap_every=5,
              seed=3)
    rows, swap = parallel_tempering(RS.SpinSystem(ucs["sc"], tuple(pt["L"]), (1, 1, 1), (0, 0, 0)), pt["T"],
                                    therm_sweeps=pt["therm"], meas_sweeps=pt["meas"], sample_every=pt["sample_every"],
                                    swap_every=pt["swap_every"], seed=pt["seed"])
    pt["rows"] = [{k: (float(v) if isinstance(v, (float, np.floating)) else v) for k, v in r.items()
                   if k in ("T", "E", "dE", "m", "dm", "C", "U4", "acceptance", "ncolors")} for r in rows]
    pt["swap"] = [float(x) for x in swap]
    models["parallel_tempering"] = pt

    # T_c estimation from rows of two sizes (synthetic rows with a Binder crossing)
    Ts = np.linspace(20.0, 40.0, 9)
    rows = []
    for Lc, slope in ((4, 0.010), (8, 0.022)):
        for T in Ts:
            x = np.tanh((31.0 - T) * slope * 10)
            rows.append(dict(L=[Lc] * 3, T=float(T), chi=float(np.exp(-((T - 30.5 - 4.0 / Lc) / 3.0) ** 2) * Lc),
                             C=float(1.0 / (1 + (T - 29.0) ** 2)), U4=float(0.55 + 0.1 * x)))
    models["mc_tc"] = dict(rows=rows, estimate=RMC.estimate_tc(rows))

    # ---------------------------------------------------------------- S(q, w) (magex/spectra.py:49-84)
    from magex import spectra as RSP

    def sqw(tag, uc, L, pbc, B, alpha, dt, T, seed, qfrac, nsteps, sample_every, nseg):
        s = RS.SpinSystem(uc, L, pbc, B)
        sol = LLGSolver(s, alpha, dt, T, seed)
        e = s.init_spins("reference")
        out[f"sqw/{tag}/e0"] = e.copy()
        E, Sp, Sl, e = RSP.structure_factor(s, sol, e, np.asarray(qfrac, float), nsteps, sample_every, nseg)
        out[f"sqw/{tag}/E"] = E
        out[f"sqw/{tag}/S_perp"] = Sp
        out[f"sqw/{tag}/S_par"] = Sl
        out[f"sqw/{tag}/e_end"] = e
        models["sqw__" + tag] = dict(L=list(L), pbc=[bool(x) for x in pbc], B=list(map(float, B)), alpha=alpha, dt=dt,
                                     T=T, seed=seed, qfrac=np.asarray(qfrac, float).tolist(), nsteps=nsteps,
                                     sample_every=sample_every, nseg=nseg)

    sqw("tri", ucs["tri"], (8, 8, 1), (1, 1, 0), (0.0, 0.0, 1.0), 0.05, 1e-3, 5.0, 13,
        [[0, 0, 0], [0.125, 0, 0], [0.25, 0, 0], [0.5, 0, 0], [1 / 3, 1 / 3, 0], [0.3, 0.1, 0]], 400, 5, 2)
    sqw("bcc2", ucs["bcc2"], (4, 4, 4), (1, 1, 1), (0.0, 0.0, 0.5), 0.1, 1e-4, 50.0, 14,
        [[0, 0, 0], [0.25, 0, 0], [0.25, 0.25, 0.25], [0.5, 0.5, 0.5], [0, 0, 0.75], [0.2, 0.35, 0.6]], 240, 4, 2)

    # ---------------------------------------------------------------- output files (magex/observables.py, llg.py)
    import hashlib
    from magex import observables as ROBS
    from magex.llg import _write_table, save_spins

    def digest(path):
        with open(path, "rb") as f:
            data = f.read()
        return dict(sha256=hashlib.sha256(data).hexdigest(), size=len(data))

    files = {}
    for tag, uc, L, pbc in (("tri", ucs["tri"], (6, 5, 1), (1, 1, 0)), ("bcc2", ucs["bcc2"], (3, 2, 2), (1, 1, 1))):
        s = RS.SpinSystem(uc, L, pbc, (0.0, 0.0, 0.5))
        e = s.init_spins("random", seed=21)
        e[0] = [1e-9, -2.5e-7, -1.0]                    # tiny and negative components exercise the formats
        out[f"out/{tag}/e"] = e
        d = {}
        for name, fn in (("xyz", lambda q: ROBS.write_xyz(q, s, e, comment="t=1.5 ps")),
                         ("vtk", lambda q: ROBS.write_vtk(q, s, e, extra=dict(E=np.linspace(-3, 4e-6, s.N)))),
                         ("ovf", lambda q: ROBS.write_ovf_atomistic(q, s, e)),
                         ("csv", lambda q: save_spins(q.replace(".csv", ".npz"), s, e))):
            q = os.path.join(tmp, f"{tag}.{name}")
            fn(q)
            d[name] = digest(q)
        files[tag] = dict(L=list(L), pbc=[bool(x) for x in pbc], files=d)
    q = os.path.join(tmp, "table.csv")
    _write_table(q, out["sc16/table"])
    files["table"] = digest(q)
    models["outputs"] = files

    # ---------------------------------------------------------------- topological charge
    s = RS.SpinSystem(ucs["tri"], (30, 30, 1), (1, 1, 0))
    c = s.positions[:, :2].mean(0)
    r = s.positions[:, :2] - c
    R = np.linalg.norm(r, axis=1)
    th = np.pi * np.exp(-(R / 8.0) ** 2)
    ph = np.arctan2(r[:, 1], r[:, 0])
    e = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)
    out["topo/skyrmion_e"] = e
    out["topo/skyrmion_Q"] = np.array(RT.topological_charge(s, e))
    e2 = s.init_spins("random", seed=11)
    out["topo/random_e"] = e2
    out["topo/random_Q"] = np.array(RT.topological_charge(s, e2))

    # the same charge on other lattices and planes, open and periodic in-plane axes (periodic Delaunay
    # of magex/texture.py:30-63): a Gaussian bubble texture and random spins
    topo_cases = {}
    ucs_topo = dict(ucs, sq=uc_of("sq", RM.make_model(lattice="square", J=[1.0], D=0.2)))
    for tag, model, L, pbc, plane, layer in (("square", "sq", (24, 24, 1), (1, 1, 0), "xy", 0),
                                             ("honeycomb", "honeycomb_bulk", (12, 12, 1), (1, 1, 0), "xy", 0),
                                             ("kagome", "kagome", (10, 10, 1), (1, 0, 0), "xy", 0),
                                             ("sc_xz", "sc", (8, 4, 8), (1, 1, 1), "xz", 2),
                                             ("sc_open", "sc", (10, 10, 3), (0, 0, 0), "xy", 1)):
        s = RS.SpinSystem(ucs_topo[model], L, pbc)
        ax, bx, _ = RT.PLANES[plane]
        r = s.positions[:, [ax, bx]] - s.positions[:, [ax, bx]].mean(0)
        R = np.linalg.norm(r, axis=1)
        th = np.pi * np.exp(-(R / (0.3 * R.max())) ** 2)
        ph = np.arctan2(r[:, 1], r[:, 0])
        e = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)
        e2 = s.init_spins("random", seed=13)
        out[f"topo2/{tag}/bubble_e"], out[f"topo2/{tag}/random_e"] = e, e2
        out[f"topo2/{tag}/bubble_Q"] = np.array(RT.topological_charge(s, e, plane, layer))
        out[f"topo2/{tag}/random_Q"] = np.array(RT.topological_charge(s, e2, plane, layer))
        topo_cases[tag] = dict(model=model, L=list(L), pbc=[bool(x) for x in pbc], plane=plane, layer=layer)
    models["topo2"] = topo_cases
    # damped-LLG relaxation of magex/minimize.py:168-181 (alpha 1, dt 2 fs, no precession, torque
    # checked every 50 steps): to a torque tolerance, with a pinned layer, and stopped by max_iter
    from magex.minimize import minimize as RMIN
    relax_cases = {}
    for tag, model, L, pbc, B, tol, max_iter, structure, seed in (
            ("tri", "tri", (12, 12, 1), (1, 1, 0), (0.0, 0.0, 1.0), 1e-4, None, None, 21),
            ("sc_pinned", "sc_dmi", (4, 4, 4), (1, 1, 0), (0.2, 0.0, 0.3), 1e-5, 20000,
             dict(pinned=[dict(region="bottom", layers=1, direction=[1, 0, 0])]), 22),
            ("max_iter", "bcc2", (3, 3, 3), (1, 1, 1), (0.0, 0.0, 0.5), 1e-12, 120, None, 23)):
        s = RS.SpinSystem(ucs_topo[model], L, pbc, B)
        if structure:
            apply_structure(s, structure)
        e0 = s.init_spins("random", seed=seed)
        e, info = RMIN(s, e0.copy(), "llg", tol=tol, max_iter=max_iter)
        out[f"relax/{tag}/e0"], out[f"relax/{tag}/e"] = e0, e
        out[f"relax/{tag}/iterations"] = np.array(info["iterations"])
        out[f"relax/{tag}/energy"] = np.array(info["energy"])
        relax_cases[tag] = dict(model=model, L=list(L), pbc=[bool(x) for x in pbc], B=list(B), tol=tol,
                                max_iter=max_iter, structure=structure)
    models["relax"] = relax_cases

    # FMR ring-down of magex/programs.py:124-150 from states relaxed to 1e-11 (so that magex's own
    # L-BFGS relaxation inside fmr returns at once)
    from magex.programs import fmr as RFMR
    fmr_cases = {}
    for tag, model, L, pbc, B, kw in (
            ("tri_heun", "tri", (8, 8, 1), (1, 1, 0), (0.0, 0.0, 1.0),
             dict(B_pulse=0.05, alpha=0.01, dt=2e-3, steps=3000, every=5)),
            ("sc_depondt", "sc_dmi", (4, 4, 4), (1, 1, 1), (0.0, 0.0, 2.0),
             dict(B_pulse=0.02, direction=(0, 1, 1), alpha=0.005, dt=1e-3, steps=2002, every=7,
                  integrator="depondt"))):
        s = RS.SpinSystem(ucs_topo[model], L, pbc, B)
        e_rel, _ = RMIN(s, s.init_spins("ferro", (0, 0, 1)), "lbfgs", tol=1e-11)
        (f, F), fpk, table = RFMR(s, e_rel.copy(), **kw)
        out[f"fmr/{tag}/e"], out[f"fmr/{tag}/f"], out[f"fmr/{tag}/F"] = e_rel, f, F
        out[f"fmr/{tag}/fpk"], out[f"fmr/{tag}/table"] = np.array(fpk), table
        fmr_cases[tag] = dict(model=model, L=list(L), pbc=[bool(x) for x in pbc], B=list(B), kw=kw)
    models["fmr"] = fmr_cases

    # the Python-API tutorial of magex (docs/tutorials/07_python_api.md:18-26): write_model ->
    # load_results -> SpinSystem -> LLGSolver.run (20,000 steps, rows every 200, 10 snapshots) -> Q
    from magex.models import write_model as RWM
    from magex.llg import LLGSolver as RLLG
    p = os.path.join(tmp, "tutorial_tri.json")
    RWM(p, lattice="triangular", J=[2.0], D=1.0, moment=3.0)
    s = RS.SpinSystem(RS.load_results(p), supercell=(48, 48, 1), pbc=(True, True, False), field=(0, 0, 2.0))
    e0 = s.init_spins("random", seed=1)
    e, table, snaps = RLLG(s, alpha=0.5, dt=2e-3, temperature=0.0).run(e0.copy(), steps=20000, output_every=200,
                                                                        snapshots=10)
    out["tutorial/e"], out["tutorial/table"] = e, table
    out["tutorial/snap_t"] = np.array([t for t, _ in snaps])
    out["tutorial/snap5"] = snaps[5][1]
    out["tutorial/Q"] = np.array(RT.topological_charge(s, e))

    # magex's own texture initialisers on a 40 x 40 triangular film (the charges of
    # tests/test_universal.py:81-91): one and two skyrmions, helicity 0 with vorticity +1 and -1
    s = RS.SpinSystem(ucs["tri"], (40, 40, 1), (1, 1, 0), (0, 0, 1.0))
    for tag, kw in (("skyrmion", dict(kind="skyrmion", radius=8.0)),
                    ("skyrmions", dict(kind="skyrmions", centers=[[30, 30], [80, 60]], radius=6.0)),
                    ("helicity0", dict(kind="skyrmion", radius=8.0, helicity=0.0)),
                    ("antiskyrmion", dict(kind="skyrmion", radius=8.0, helicity=0.0, vorticity=-1))):
        e = s.init_spins(**kw)
        out[f"topo3/{tag}_e"] = e
        out[f"topo3/{tag}_Q"] = np.array(RT.topological_charge(s, e, "xy", 0))

    np.savez_compressed(os.path.join(HERE, "llg_golden.npz"), **out)
    with open(os.path.join(HERE, "models.json"), "w") as f:
        json.dump(models, f)
    print("wrote", os.path.join(HERE, "llg_golden.npz"), os.path.join(HERE, "models.json"))


def _thermal_bcc2_run(ref_root, th, seed):
    """One Langevin run of magex's LLGSolver on the config-2 Hamiltonian: E/N and |M| samples."""
    sys.path.insert(0, ref_root)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from magex import spinmodel as RS
    from magex.llg import LLGSolver
    from magex_gb300.workloads import bcc_two_site_model
    tmp = tempfile.mkdtemp()
    path = os.path.join(tmp, "bcc2.json")
    with open(path, "w") as f:
        json.dump(bcc_two_site_model(J=(20.0, 10.0, -1.0), seed=0), f)
    s = RS.SpinSystem(RS.load_results(path), (th["L"],) * 3, (1, 1, 1), (0.0, 0.0, th["Bz"]))
    sol = LLGSolver(s, alpha=th["alpha"], dt=th["dt"], temperature=th["T"], seed=seed)
    e = s.init_spins("ferro")
    for _ in range(th["equil"]):
        e = sol.step(e)
    Es, Ms = [], []
    for k in range(th["sample"]):
        e = sol.step(e)
        if k % th["every"] == th["every"] - 1:
            Es.append(s.energy(e, per_spin=True))
            Ms.append(np.linalg.norm(e.mean(0)))
    return np.array(Es), np.array(Ms)


def thermal_bcc2(ref_root):
    """Equilibrium statistics of the benchmark Hamiltonian from magex's own Langevin runs.

    Two-site bcc 8^3 (1,024 spins), shells 8+6+12 with per-bond full 3x3 tensors (isotropic
    20/10/-1 meV, 1 % symmetric anisotropic part, DMI |D| = 1 meV), SIA K = 0.01 meV along z,
    B = (0, 0, 0.5) T, T = 300 K, alpha 0.05, dt 0.1 fs: `nruns` independent LLGSolver runs (NumPy
    Heun, noise default_rng(seed).normal per step, magex/llg.py:106-122,216-227; seeds seed0,
    seed0 + 1, ...) from the ferromagnetic state, `equil` steps discarded, then E/N
    (magex/spinmodel.py:475-484) and |M| = |mean e| sampled every `every` steps over `sample` steps.

    Each run gives one mean per observable.  The energy has slow components (its autocorrelation
    still reads a few per cent after 10,000 steps), so 20-block errors of one run understate the
    scatter between runs; the standard error used is that of the run means (sem_runs), together
    with the scatter of one run (sd_run), which a run of the same length on the GPU shares."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    import scipy

    th = dict(L=8, alpha=0.05, dt=1e-4, T=300.0, Bz=0.5, seed0=31, nruns=8, equil=20000, sample=200000, every=20,
              model="bcc2", model_kwargs=dict(J=[20.0, 10.0, -1.0], seed=0))
    seeds = [th["seed0"] + k for k in range(th["nruns"])]
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    with ProcessPoolExecutor(max_workers=min(8, len(seeds)), mp_context=mp.get_context("spawn")) as ex:
        runs = list(ex.map(_thermal_bcc2_run, [ref_root] * len(seeds), [th] * len(seeds), seeds))
    out = {"numpy_version": np.array(np.__version__), "scipy_version": np.array(scipy.__version__),
           "params": np.array(json.dumps(th)), "E_series0": runs[0][0], "M_series0": runs[0][1]}
    for key, col in (("E", 0), ("M", 1)):
        means = np.array([r[col].mean() for r in runs])
        out[f"{key}_run_means"] = means
        out[f"{key}_mean"] = np.array(means.mean())
        out[f"{key}_sd_run"] = np.array(means.std(ddof=1))
        out[f"{key}_sem"] = np.array(means.std(ddof=1) / np.sqrt(len(means)))
    np.savez_compressed(os.path.join(HERE, "thermal_bcc2.npz"), **out)
    print("wrote", os.path.join(HERE, "thermal_bcc2.npz"),
          {k: out[k].tolist() for k in ("E_mean", "E_sem", "E_sd_run", "M_mean", "M_sem", "M_sd_run")})


def adversarial(ref_root):
    """T = 0 trajectories of models built to stress a fixed-point exchange sum (adversarial.npz).

    sc_decades: simple cubic 6^3 with three shells J = 100, 1e-3 and 1e-6 meV (eight decades in one
    stencil), nearest-neighbour DMI 5 meV and an anisotropic part of 1e-2 meV, a near-zero single-ion
    constant K = 1e-9 meV, |B| = 100 T along an oblique axis.  bcc2_decades: two-site bcc 4^3, four
    shells 20 / 10 / -1 / 1e-6 meV with per-shell full tensors (1 % anisotropic, DMI 5 %), K = 1e-10
    meV, the same 100 T field.  The models are read with jtol = 1e-12 (magex's default 1e-4 would drop the
    1e-6 meV shells).  magex's LLGSolver (NumPy Heun, magex/llg.py:216-227), alpha 0.1,
    dt 0.1 fs, 1000 steps from random spins; spins kept after 1, 10, 100 and 1000 steps, final
    energy and effective field."""
    sys.path.insert(0, ref_root)
    import scipy
    from magex import models as RM
    from magex import spinmodel as RS
    from magex.llg import LLGSolver
    from magex_gb300.workloads import bcc_two_site_model

    B = 100.0 * np.array([0.3, -0.6, 0.75]) / np.linalg.norm([0.3, -0.6, 0.75])
    cases = {
        "sc_decades": (RM.make_model(lattice="sc", J=[100.0, 1e-3, 1e-6], D=5.0,
                                     Jani=[[1e-2, 0, 0], [0, -2e-2, 0], [0, 0, 1e-2]], K=1e-9, moment=2.0),
                       (6, 6, 6)),
        "bcc2_decades": (bcc_two_site_model(J=(20.0, 10.0, -1.0, 1e-6), dmi_frac=0.05, per="shell", K=1e-10, seed=5),
                         (4, 4, 4)),
    }
    tmp = tempfile.mkdtemp()
    out = {"numpy_version": np.array(np.__version__), "scipy_version": np.array(scipy.__version__)}
    meta = {}
    keep = (1, 10, 100, 1000)
    for tag, (d, L) in cases.items():
        path = os.path.join(tmp, tag + ".json")
        with open(path, "w") as f:
            json.dump(d, f)
        s = RS.SpinSystem(RS.load_results(path, jtol=1e-12), L, (1, 1, 1), tuple(B))
        e = s.init_spins("random", seed=11)
        sol = LLGSolver(s, 0.1, 1e-4, 0.0, 1)
        out[f"{tag}/e0"] = e.copy()
        for n in range(1, keep[-1] + 1):
            e = sol.step(e)
            if n in keep:
                out[f"{tag}/e{n}"] = e.copy()
        out[f"{tag}/energy"] = np.array(s.energy(e))
        out[f"{tag}/field"] = s.effective_field(e)
        meta[tag] = dict(model=d, L=list(L), B=list(map(float, B)), alpha=0.1, dt=1e-4, keep=list(keep), jtol=1e-12,
                         ncouplings=len(s.bonds) if hasattr(s, "bonds") else None)
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "adversarial.npz"), **out)
    print("wrote", os.path.join(HERE, "adversarial.npz"))


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else "/root/reference"
    if "--thermal-bcc2" in sys.argv:
        thermal_bcc2(root)
    elif "--adversarial" in sys.argv:
        adversarial(root)
    else:
        main(root)
