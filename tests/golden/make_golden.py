"""Extract the reference's regression fixtures used to pin the oracle.

Reads ``samples/<Case>/reference.out`` from a checkout of magic-sph/pizza
(the tree given by --ref, read only) and writes the rows that come
from the collocation runs into ``tests/golden/<Case>.txt``, together with the
namelist values of the run that produced them (``tests/golden/cases.json``).

Rows kept per case (the fixture concatenates several chained runs; only the
first run starts from the namelist and needs no checkpoint):
  NonRotRa2e3       all 11 rows   (e_kin, coll smat CNAB2, non-rotating)
  RotE1e3EkPump     rows 0-10     (e_kin_3D, coll smat CNAB2, Ekman pumping)
  MultistepSchemes  rows 0-200    (e_kin_3D, coll smat SBDF3 + CNAB2 bridge)
  TimeStepChange    all 21 rows   (e_kin, coll dmat SBDF3, CFL dt changes)
  DIRKSchemes       rows 0-10     (e_kin_3D, coll smat ARS222, a DIRK scheme)
  RotInteg          rows 0-200    (e_kin_3D, integ smat CNAB2, tau boundary rows)
  RotIntegContinue  rows 201-216  (e_kin_3D, RotInteg's second run: its first run's
                                   final state read onto n_r_max=97, m_max=64, integ
                                   dmat SBDF3 with the CNAB2 bridge and AB1)
  FingConv          rows 0-5      (e_kin, fingering convection: temperature and
                                   composition, non-rotating integ smat SBDF3)
  FingConvContinue  rows 6-11     (e_kin, FingConv's second run: its first run's final
                                   state read onto the n_r_max=33 collocation grid,
                                   DIRK BPR353)

A case with "restart_from" starts from the final state of that case's run
(written as a checkpoint and read back) instead of its own start fields;
"skip" is the number of fixture lines before its rows.
"""
import argparse
import json
import os

CASES = {
    "NonRotRa2e3": dict(
        rows=11, series="e_kin",
        params=dict(n_r_max=33, n_cheb_max=33, m_max=32, n_time_steps=1000, dtMax=1e-3,
                    l_non_rot=True, ra=2.0e3, pr=1.0, ek=1.0e-3, radratio=0.35,
                    g0=1.0, g1=0.0, g2=0.0, init_t=3, amp_t=2.5e-4, n_log_step=100)),
    "RotE1e3EkPump": dict(
        rows=11, series="e_kin_3D",
        params=dict(n_r_max=32, n_cheb_max=32, m_max=32, n_time_steps=1000, dtMax=1e-4,
                    ra=2.77e4, pr=1.0, ek=1.0e-3, radratio=0.35, g0=0.0, g1=1.0, g2=0.0,
                    l_ek_pump=True, init_t=4, amp_t=2.5e-4, n_log_step=100)),
    "MultistepSchemes": dict(
        rows=201, series="e_kin_3D",
        params=dict(n_r_max=32, n_cheb_max=32, m_max=32, n_time_steps=200, dtMax=1e-4,
                    time_scheme="SBDF3", ra=4.0e4, pr=1.0, ek=1.0e-3, radratio=0.35,
                    g0=0.0, g1=1.0, g2=0.0, l_ek_pump=True, init_t=4, amp_t=2.5e-4,
                    n_log_step=1)),
    "TimeStepChange": dict(
        rows=21, series="e_kin",
        params=dict(n_r_max=48, n_cheb_max=48, m_max=64, n_time_steps=2000, dtMax=5e-4,
                    time_scheme="SBDF3", courfac=2.5, l_non_rot=True,
                    matrix_solve="INFLUENCE", ra=1.0e4, pr=1.0, ek=1.0e-3, radratio=0.35,
                    g0=1.0, g1=0.0, g2=0.0, init_t=-1, amp_t=1.0e-2, n_log_step=100)),
    "DIRKSchemes": dict(
        rows=11, series="e_kin_3D",
        params=dict(n_r_max=33, n_cheb_max=33, m_max=32, n_time_steps=100, dtMax=1e-5,
                    time_scheme="ARS222", courfac=1.0, ra=6.0e4, pr=1.0, ek=1.0e-3,
                    radratio=0.35, g0=0.0, g1=1.0, g2=0.0, l_ek_pump=False, init_t=4,
                    amp_t=2.5e-4, n_log_step=10)),
    "RotInteg": dict(
        rows=201, series="e_kin_3D",
        params=dict(n_r_max=49, n_cheb_max=32, m_max=32, n_time_steps=4000, dtMax=1e-1,
                    cheb_method="INTEG", matrix_solve="DIRECT", l_rerror_fix=True, rerror_fac=5e2,
                    courfac=4.0, time_scale="ROT", ra=5.0e4, pr=1.0, ek=1.0e-3, radratio=0.35,
                    g0=0.0, g1=1.0, g2=0.0, ktopv=2, kbotv=2, l_ek_pump=False, init_t=-1,
                    amp_t=1.0e-2, n_log_step=20)),
    "RotIntegContinue": dict(
        rows=16, skip=201, series="e_kin_3D", restart_from="RotInteg",
        params=dict(n_r_max=97, n_cheb_max=64, m_max=64, n_time_steps=300, dtMax=1e-1,
                    cheb_method="INTEG", matrix_solve="INFLUENCE", corio_term="EXPLICIT",
                    l_rerror_fix=True, rerror_fac=5e2, courfac=4.0, time_scale="ROT", time_scheme="SBDF3",
                    ra=2.0e6, pr=1.0, ek=1.0e-4, radratio=0.35, g0=0.0, g1=1.0, g2=0.0, ktopv=2, kbotv=2,
                    l_ek_pump=True, n_log_step=20)),
    "FingConv": dict(
        rows=6, series="e_kin",
        params=dict(n_r_max=49, n_cheb_max=32, m_max=32, n_time_steps=500, dtMax=1e-3, l_non_rot=True,
                    cheb_method="INTEG", time_scheme="SBDF3", ra=-1.0e4, pr=0.3, raxi=2.0e4, sc=3.0,
                    ek=1.0e-3, radratio=0.35, g0=1.0, g1=0.0, g2=0.0, ktopt=1, kbott=1, ktopxi=1,
                    kbotxi=1, ktopv=2, kbotv=2, init_t=-1, amp_t=2.5e-4, init_xi=0, amp_xi=2.5e-4,
                    n_log_step=100)),
    "FingConvContinue": dict(
        rows=6, skip=6, series="e_kin", restart_from="FingConv",
        params=dict(n_r_max=33, n_cheb_max=33, m_max=32, n_time_steps=500, dtMax=1e-3, l_non_rot=True,
                    cheb_method="COLL", time_scheme="BPR353", ra=-1.0e4, pr=0.3, raxi=2.0e4, sc=3.0,
                    ek=1.0e-3, radratio=0.35, g0=1.0, g1=0.0, g2=0.0, ktopt=1, kbott=1, ktopxi=1,
                    kbotxi=1, ktopv=2, kbotv=2, n_log_step=100)),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the pizza source tree (read only)")
    args = ap.parse_args()
    here = os.path.dirname(os.path.abspath(__file__))
    meta = {}
    for case, spec in CASES.items():
        sample = spec.get("restart_from", case)
        src = os.path.join(args.ref, "samples", sample, "reference.out")
        with open(src) as f:
            lines = [ln for ln in f.read().splitlines() if ln.strip()]
        skip = spec.get("skip", 0)
        keep = lines[skip:skip + spec["rows"]]
        with open(os.path.join(here, f"{case}.txt"), "w") as f:
            f.write("\n".join(keep) + "\n")
        meta[case] = dict(series=spec["series"], rows=spec["rows"], params=spec["params"],
                          source=f"samples/{sample}/reference.out")
        if "restart_from" in spec:
            meta[case]["restart_from"] = spec["restart_from"]
            meta[case]["skip"] = skip
    with open(os.path.join(here, "cases.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
