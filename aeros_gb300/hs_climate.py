"""Held-Suarez climate run and its zonal-mean summary (the long-run check).

  python -m aeros_gb300.hs_climate --trunc 42 --nlev 20 --days 1200 --spinup 200 \\
      --members 4 --precision fp64|split [--json FILE]

The run follows the reference's Held-Suarez driver: start from rest at
T = 264 K and ps = 1000 hPa plus N(0, 0.1^2) K noise on the grid temperature
(one seed per member), integrate `days` days with dt = 1800 s, and take daily
samples of the zonal-mean statistics (src/aeros_diagnostics.f90:153-276) over
the last days - spinup days.  The summary reports the quantities of the
reference's regression table: jet maxima of [u], surface [u], the maxima of
[v'T'], [u'v'], eddy kinetic energy and [T'^2], the surface equator-pole [T]
contrast and the hemispheric asymmetry of [u].  Level pressures are
sigma * 1000 hPa.  Statistics are computed on the member-mean fields; the
member spread of the jet maximum measures the sampling noise.
"""
import argparse
import json
import sys
import time

import numpy as np


def initial_states(dyn, sht, seed0):
    dyn.set_isothermal(264.0, 1.0e5)
    vor, div, t, lnps = dyn.get_state(squeeze=False)
    t = t.copy()
    for e in range(dyn.nmember):
        rng = np.random.default_rng(seed0 + e)
        t[e] = sht.analysis(sht.synthesis(t[e]) + rng.normal(0.0, 0.1, (dyn.nlev, dyn.nlat, dyn.nlon)))
    dyn.set_state(vor, div, t, lnps)


def _argmax2(f):
    k, j = np.unravel_index(np.argmax(f), f.shape)
    return float(f[k, j]), int(k), int(j)


def summarize(fields, lat, p_hpa):
    """Reference-table quantities from member-mean zonal statistics."""
    u, vt, uv, eke, tvar, T = (fields[k] for k in ("u", "vt", "uv", "eke", "tvar", "temp"))
    nh, sh = lat > 0, lat < 0
    out = {}
    for name, mask in (("jet_nh", nh), ("jet_sh", sh)):
        v, k, j = _argmax2(np.where(mask[None, :], u, -np.inf))
        out[name] = {"u_max": v, "lat": float(lat[j]), "p_hpa": float(p_hpa[k])}
    us = fields["u_sfc"]
    j = int(np.argmax(us))
    out["u_surface_max"] = {"u": float(us[j]), "lat": float(lat[j])}
    trop = np.abs(lat) < 15.0
    out["u_surface_tropics_min"] = float(np.min(us[trop]))
    for name, f in (("vT_max", vt), ("uv_max", uv)):
        v, k, j = _argmax2(f)
        out[name] = {"value": v, "lat": float(lat[j]), "p_hpa": float(p_hpa[k])}
    out["eke_max"] = float(np.max(eke))
    out["tvar_max"] = float(np.max(tvar))
    ts = T[-1]
    out["t_surface_equator"] = float(np.max(ts))
    out["t_surface_pole"] = float(np.min(ts))
    out["t_surface_contrast"] = float(np.max(ts) - np.min(ts))
    out["u_hemispheric_asymmetry"] = float(np.linalg.norm(u - u[:, ::-1]) / np.linalg.norm(u))
    return out


def run(trunc=42, nlev=20, days=1200, spinup=200, members=4, precision="fp64", seed0=0):
    from .params import held_suarez_params, PREC_FP64, PREC_SPLIT
    from .dynamics import AerosDyn
    from .spectral import AerosSHT
    p = held_suarez_params(trunc=trunc, nlev=nlev, nmember=members,
                           precision=PREC_SPLIT if precision == "split" else PREC_FP64)
    dyn = AerosDyn(p)
    sht = AerosSHT(trunc, batch_max=nlev)
    initial_states(dyn, sht, seed0)
    spd = int(round(86400.0 / p.dt))
    t0 = time.perf_counter()
    dyn.step(spinup * spd)
    for _ in range(days - spinup):
        dyn.step(spd)
        dyn.diag_accumulate()
    wall = time.perf_counter() - t0
    stats = [dyn.diag_read(e) for e in range(members)]
    keys = ("u", "v", "temp", "uv", "vt", "eke", "tvar", "ps", "u_sfc")
    mean = {k: np.mean([s[k] for s in stats], axis=0) for k in keys}
    lat = np.degrees(np.arcsin(dyn.sinlat))
    p_hpa = dyn.sigma_full * 1000.0
    res = summarize(mean, lat, p_hpa)
    jets = [summarize({k: s[k] for k in keys}, lat, p_hpa)["jet_nh"]["u_max"] for s in stats]
    res["jet_nh_member_spread"] = float(np.std(jets))
    res["config"] = {"trunc": trunc, "nlev": nlev, "days": days, "averaged_days": days - spinup,
                     "members": members, "precision": precision, "seed0": seed0, "nsample": stats[0]["nsample"]}
    res["wall_s"] = wall
    res["sypd_aggregate"] = members * days / 365.25 / (wall / 86400.0)
    return res


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--trunc", type=int, default=42)
    ap.add_argument("--nlev", type=int, default=20)
    ap.add_argument("--days", type=int, default=1200)
    ap.add_argument("--spinup", type=int, default=200)
    ap.add_argument("--members", type=int, default=4)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "split"])
    ap.add_argument("--seed0", type=int, default=0)
    ap.add_argument("--json", default=None)
    a = ap.parse_args(argv)
    res = run(a.trunc, a.nlev, a.days, a.spinup, a.members, a.precision, a.seed0)
    txt = json.dumps(res)
    print(txt)
    if a.json:
        with open(a.json, "w") as f:
            f.write(txt + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
