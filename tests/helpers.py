"""Shared helpers of the test-suite: rebuild the golden systems with the GB300 host model."""
import numpy as np

from magex_gb300.lattice import Supercell
from magex_gb300.spinmodel import load_results


def golden_supercell(golden_models, tag):
    """Supercell + trajectory metadata of golden trajectory `tag` (structure edits applied)."""
    meta = golden_models["traj__" + tag]
    model_name = {
        "sc16": "sc", "sc6_thermal": "sc_dmi", "bcc2_thermal": "bcc2", "bcc2_T0": "bcc2", "bcc2_shell4": "bcc2_shell4",
        "tri16": "tri", "sc_depondt": "sc_dmi", "tri_depondt_thermal": "tri", "sc_open": "sc_open",
        "sc_tiny_fold": "sc_two_shell", "sc_afm": "sc_afm", "honeycomb": "honeycomb_bulk", "sc_structure": "sc_dmi",
        "sc_cubic": "sc_dmi", "tri_cubic_thermal": "tri",
    }[tag]
    uc = load_results(golden_models[model_name]["model"])
    sc = Supercell(uc, meta["L"], meta["pbc"], meta["B"])
    if meta.get("structure"):
        apply_structure_subset(sc, meta["structure"])
    return sc, meta


def apply_structure_subset(sc, st):
    """The parts of magex.structure.apply_structure that the golden case uses (magex/structure.py):
    one bulk material with alpha and T (:172-179), a pinned bottom layer with a direction (:198-207)
    and a linear temperature profile along x that fills sites without a material T (:208-225)."""
    for m in st.get("materials", []):
        if "Kc" in m:                     # magex/structure.py:163-165,190-191 (one material covers every site)
            axes = m.get("cubic_axes")
            sc.cubic = (np.full(sc.N, float(m["Kc"])), np.eye(3) if axes is None else np.asarray(axes, float))
        if "K2" in m or "K3" in m:        # magex/structure.py:166-169,192-193 and magex/terms.py:59-63
            u = np.asarray(m.get("K_axis", (0, 0, 1)), float)
            sc.uniaxial_higher = (np.full(sc.N, float(m.get("K2", 0.0))), np.full(sc.N, float(m.get("K3", 0.0))),
                                  u / np.linalg.norm(u))
        if "alpha" in m:
            sc.alpha_site = np.full(sc.N, float(m["alpha"]))
        if "T" in m:
            sc.site_T = np.full(sc.N, float(m["T"]))
    cells = np.repeat(np.stack(np.meshgrid(*[np.arange(n) for n in sc.L], indexing="ij"), -1).reshape(-1, 3), sc.ns, 0)
    for p in st.get("pinned", []):
        n = int(p.get("layers", 1))
        z = cells[:, 2]
        sel = z < z.min() + n
        if sc.pinned is None:
            sc.pinned = np.zeros(sc.N, bool)
            sc.pinned_dir = sc.ref.copy()
        sc.pinned |= sel
        if "direction" in p:
            d = np.asarray(p["direction"], float)
            sc.pinned_dir[sel] = d / np.linalg.norm(d)
    tp = st.get("temperature_profile")
    if tp:
        P = sc.positions
        u = (P[:, 0] - P[:, 0].min()) / max(np.ptp(P[:, 0]), 1e-9)
        prof = float(tp["T0"]) + (float(tp["T1"]) - float(tp["T0"])) * u
        sc.site_T = prof if sc.site_T is None else np.where(np.isnan(sc.site_T), prof, sc.site_T)
    return sc


def golden_irregular(golden, golden_models, tag):
    """NeighbourList of a golden carved / exchange-edited system, built from the reference's stored
    3N x 3N coupling matrix and per-site arrays (A, mu, signs, pinned, site T, damping)."""
    import scipy.sparse as sp
    from magex_gb300.lattice import NeighbourList
    meta = golden_models["irregular__" + tag]
    N = meta["N"]
    J = sp.csr_matrix((golden[f"{tag}/Jsp_data"], golden[f"{tag}/Jsp_indices"], golden[f"{tag}/Jsp_indptr"]),
                      shape=(3 * N, 3 * N))
    nl = NeighbourList.from_matrix(J, golden[f"{tag}/mu"], golden[f"{tag}/A"], golden[f"{tag}/signs"], meta["B"])
    for name in ("pinned", "site_T", "alpha_site"):
        if f"{tag}/{name}" in golden.files:
            setattr(nl, name, np.array(golden[f"{tag}/{name}"]))
    return nl, meta, J


def thermal_system(golden, golden_models):
    """The sc ferromagnet of the reference's thermal-equilibrium fixture and its run parameters."""
    import json
    th = json.loads(str(golden["thermal/params"]))
    sc = Supercell(load_results(golden_models["sc"]["model"]), (th["L"],) * 3, (True, True, True),
                   (0.0, 0.0, th["Bz"]))
    return sc, th


def block_stats(x, nblocks=20):
    """Mean of a time series and the standard error of the mean from nblocks block averages."""
    x = np.asarray(x, float)
    b = x[: len(x) // nblocks * nblocks].reshape(nblocks, -1).mean(1)
    return float(b.mean()), float(b.std(ddof=1) / np.sqrt(nblocks))


def assert_within_3_sigma(golden, key, mean, sem):
    ref, ref_sem = float(golden[f"thermal/{key}_mean"]), float(golden[f"thermal/{key}_sem"])
    bound = 3.0 * np.hypot(ref_sem, sem)
    assert abs(mean - ref) <= bound, (key, mean, ref, bound)


UC_OF = {"gauss_dmi": "sc_dmi", "uniform_sc": "sc", "heatbath_tri": "tri", "hinzke_bcc2": "bcc2",
         "T0_afm": "sc_afm", "open_kagome": "kagome", "structure": "sc_dmi", "bcc2_shell4": "bcc2_shell4",
         "cubic": "sc_dmi", "cubic_heatbath": "sc_dmi"}
MC_TAGS = list(UC_OF) + ["sphere"]


def mc_system(golden, golden_models, tag):
    """The system of a golden Monte Carlo case (Supercell, or NeighbourList for the carved sphere)."""
    from magex_gb300.lattice import Supercell
    from magex_gb300.spinmodel import load_results
    meta = golden_models["mc__" + tag]
    if tag == "sphere":
        nl, _, _ = golden_irregular(golden, golden_models, "sc_sphere")
        return nl, meta
    sc = Supercell(load_results(golden_models[UC_OF[tag]]["model"]), tuple(meta["L"]), tuple(meta["pbc"]),
                   tuple(meta["B"]))
    if meta["structure"]:
        apply_structure_subset(sc, meta["structure"])
    return sc, meta


def callable_fields(p):
    """field_func(t) and extra_field(e) of the callables fixtures, from their stored parameters: a
    uniform field with a pulse that ends at t0 (the FMR kick of magex/programs.py:131) plus a rotating
    component, and a state-dependent per-site field (the extra_field hook of magex/sld.py:171)."""
    pulse, t0, amp, w = np.asarray(p["pulse"], float), float(p["t0"]), float(p["amp"]), float(p["w"])
    k, c = np.asarray(p["k"], float), float(p["c"])

    def field_func(t):
        f = np.array([0.0, amp * np.sin(w * t), 0.0])
        return f + pulse if t < t0 else f

    def extra_field(e):
        return c * np.cross(e, k) + 0.5 * c * e[:, [1, 2, 0]]

    return field_func, extra_field


def site_field_func(p, N):
    """A field_func(t) that returns an (N, 3) field (magex allows either shape, magex/llg.py:87): a
    fixed site pattern times a slow oscillation."""
    amp, w = float(p["amp"]), float(p["w"])
    pattern = np.linspace(-1.0, 1.0, N)[:, None] * np.array([0.5, -0.2, 0.3])

    def field_func(t):
        return amp * np.cos(w * t) * pattern

    return field_func
