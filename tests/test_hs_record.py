"""The committed 1200-day Held-Suarez T42L20 record (the long-run oracle,
profiles/held_suarez_T42L20_1200d.md) against the reference's regression
table (docs/m1_results.md:117-128 of the reference; aeros' own one-member
run), within the sampling noise the record itself shows: the FP64 ensembles
of two seed sets and the split-precision ensemble must each sit near the
reference, and split must differ from FP64 by no more than two FP64 seed sets
differ from each other (plus the member spread)."""
import json
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REC = os.path.join(ROOT, "profiles", "held_suarez_T42L20_1200d.md")

# docs/m1_results.md:117-128, T42L20 column
REF = {"jet_nh": 32.4, "jet_sh": 32.9, "jet_lat": 46.0, "u_sfc_tropics": -8.7, "vT": 21.1, "vT_lat": 37.7,
       "uv": 75.7, "uv_lat": 34.9, "eke": 367.0, "tvar": 40.4, "t_contrast": 42.2}


def records():
    with open(REC) as f:
        txt = f.read()
    block = txt.split("```json", 1)[1].split("```", 1)[0]
    out = {}
    for line in block.strip().splitlines():
        r = json.loads(line)
        c = r["config"]
        out[(c["precision"], c["seed0"])] = r
    return out


def test_record_has_every_run_and_field():
    recs = records()
    assert set(recs) == {("fp64", 0), ("split", 0), ("fp64", 100)}
    for r in recs.values():
        c = r["config"]
        assert (c["trunc"], c["nlev"], c["days"], c["averaged_days"], c["members"]) == (42, 20, 1200, 1000, 4)
        assert c["nsample"] == 1000
        for k in ("jet_nh", "jet_sh", "u_surface_max", "u_surface_tropics_min", "vT_max", "uv_max", "eke_max",
                  "tvar_max", "t_surface_contrast", "u_hemispheric_asymmetry", "jet_nh_member_spread"):
            assert k in r, k


@pytest.mark.parametrize("run", [("fp64", 0), ("split", 0), ("fp64", 100)])
def test_record_matches_reference_climate(run):
    r = records()[run]
    grid = 180.0 / 64 + 0.1          # one Gaussian latitude row
    for key, ref in (("jet_nh", REF["jet_nh"]), ("jet_sh", REF["jet_sh"])):
        assert abs(r[key]["u_max"] - ref) < 2.0
        assert abs(abs(r[key]["lat"]) - REF["jet_lat"]) <= grid
        assert 200.0 < r[key]["p_hpa"] < 260.0
    assert abs(r["u_surface_tropics_min"] - REF["u_sfc_tropics"]) < 0.5
    assert abs(r["vT_max"]["value"] - REF["vT"]) / REF["vT"] < 0.05
    assert abs(r["vT_max"]["lat"] - REF["vT_lat"]) <= grid and r["vT_max"]["p_hpa"] > 800.0
    assert abs(r["uv_max"]["value"] - REF["uv"]) / REF["uv"] < 0.10
    assert abs(r["uv_max"]["lat"] - REF["uv_lat"]) <= grid
    assert abs(r["eke_max"] - REF["eke"]) / REF["eke"] < 0.05
    assert abs(r["tvar_max"] - REF["tvar"]) / REF["tvar"] < 0.05
    assert abs(r["t_surface_contrast"] - REF["t_contrast"]) < 1.0
    assert r["u_hemispheric_asymmetry"] < 0.1


def test_split_within_fp64_sampling_noise():
    recs = records()
    a, b, s = recs[("fp64", 0)], recs[("fp64", 100)], recs[("split", 0)]
    spread = max(r["jet_nh_member_spread"] for r in recs.values())
    for key in ("jet_nh", "jet_sh"):
        noise = abs(a[key]["u_max"] - b[key]["u_max"])
        assert abs(s[key]["u_max"] - a[key]["u_max"]) <= 2 * noise + spread
    for key in ("vT_max", "uv_max"):
        noise = abs(a[key]["value"] - b[key]["value"])
        assert abs(s[key]["value"] - a[key]["value"]) <= 2 * noise + 0.05 * a[key]["value"]
    for key in ("eke_max", "tvar_max", "t_surface_contrast"):
        noise = abs(a[key] - b[key])
        assert abs(s[key] - a[key]) <= 2 * noise + 0.03 * abs(a[key])
