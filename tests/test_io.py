"""pizza's time-series text format and version-7 checkpoint layout
(pizza_gb300/pizza_io.py), on the CPU."""
import os

import numpy as np
import pytest

from pizza_gb300 import pizza_io
from pizza_gb300.pizza_io import fortran_es, format_series_line, read_checkpoint, write_checkpoint, _grid_r

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("case", ["RotE1e3EkPump", "DIRKSchemes", "NonRotRa2e3", "MultistepSchemes"])
def test_series_format_reproduces_pizza_lines(case):
    """Every line pizza.exe printed, re-printed from its values, is identical."""
    with open(os.path.join(HERE, "golden", f"{case}.txt")) as f:
        lines = [ln.rstrip("\n") for ln in f if ln.strip()]
    for ln in lines:
        vals = [float(v) for v in ln.split()]
        assert format_series_line(vals) == ln


def test_fortran_es_edge_cases():
    assert fortran_es(0.0, 16, 8) == "  0.00000000E+00"
    assert fortran_es(-1.5e-7, 16, 8) == " -1.50000000E-07"
    assert fortran_es(2.5e123, 16, 8) == "  2.50000000+123"
    assert fortran_es(1.0, 20, 12) == "  1.000000000000E+00"


def test_checkpoint_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    N, m_max = 17, 8
    M = m_max + 1

    def c():
        return rng.standard_normal((M, N)) + 1j * rng.standard_normal((M, N))

    header = dict(time=0.125, family="MULTISTEP", nexp=3, nimp=1, nold=3, dt=np.array([1e-4, 2e-4, 3e-4]),
                  ra=1e5, pr=1.0, ek=1e-3, radratio=0.35, n_r_max=N, m_max=m_max, minc=1, n_max=N,
                  r=_grid_r(N, 0.35))
    fields = dict(us=c(), up=c(), temp=c(), hist_P=[c() for _ in range(4)], hist_T=[c() for _ in range(4)])
    p = str(tmp_path / "checkpoint_end.test")
    write_checkpoint(p, header, fields)
    # header bytes as written by write_checkpoint_mloc, then us and (1 + 4) each for up and temp
    hdr = 4 + 8 + 4 + 10 + 12 + 8 * 3 + 8 * 7 + 12 + 72 + 8 + 16 + 8 * N + 12
    assert os.path.getsize(p) == hdr + 11 * M * N * 16
    ck = read_checkpoint(p)
    h = ck["header"]
    assert h["family"] == "MULTISTEP" and (h["nexp"], h["nimp"], h["nold"]) == (3, 1, 3)
    assert np.array_equal(h["dt"], header["dt"]) and h["time"] == 0.125 and h["rscheme"] == "cheb"
    for k in ("us", "up", "temp"):
        assert np.array_equal(ck[k], fields[k])
    for k in ("hist_P", "hist_T"):
        assert all(np.array_equal(a, b) for a, b in zip(ck[k], fields[k]))


def test_frame_matches_reference_reader_fixture(tmp_path):
    """write_frame's bytes equal the committed golden frame, whose contents
    the reference's own reader (python/pizza/frame.py) parsed back to the
    sample header and field (tests/golden/make_frame_golden.py)."""
    import json
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_frame_golden import sample
    header, field = sample()
    p = tmp_path / "frame.bin"
    pizza_io.write_frame(str(p), header, field)
    golden = os.path.join(os.path.dirname(__file__), "golden")
    with open(os.path.join(golden, "frame_sample.bin"), "rb") as f:
        assert p.read_bytes() == f.read()
    with open(os.path.join(golden, "frame_sample.json")) as f:
        ref = json.load(f)
    assert (ref["version"], ref["n_r_max"], ref["n_m_max"], ref["m_max"], ref["minc"], ref["n_phi_max"]) == \
        (2, 9, 5, 4, 1, 12)
    for k in ("time", "ra", "ek", "pr", "radratio", "sc", "raxi"):
        assert ref[k] == header[k]
    assert np.array_equal(np.array(ref["radius"]), header["r"])
    assert np.array_equal(np.array(ref["field_re"]) + 1j * np.array(ref["field_im"]), field)
    back = pizza_io.read_frame(str(p))
    assert np.array_equal(back["field"], field) and back["time"] == header["time"]
    assert np.array_equal(back["idx2m"], np.arange(5))


def test_spectrum_line_format():
    """'(I5, 5ES16.8)' lines with round_off (src/spectra.f90:351-360)."""
    lines = pizza_io.format_spectrum_lines(np.array([[1.5e-3, 2.0, 1e-16, -3.25e-7], [0.0, 1.0, 2.0, 3.0]]), minc=1)
    assert lines[0] == "    0  1.50000000E-03  2.00000000E+00  0.00000000E+00 -3.25000000E-07  0.00000000E+00"
    assert lines[1].startswith("    1  0.00000000E+00  1.00000000E+00")
    assert all(len(x) == 5 + 5 * 16 for x in lines)


def test_spectra_average_closed_form(tmp_path):
    """The getMSD2 recursion (useful.f90:263-293) against its closed form: the
    dt-weighted mean and standard deviation over the averaging time, dt_1 = T_1."""
    rng = np.random.default_rng(5)
    n_m, n = 7, 9
    T = np.cumsum(rng.uniform(1e-4, 3e-4, n))
    X = rng.uniform(0.0, 2.0, (n, n_m, 5))
    avg = pizza_io.SpectraAverage(n_m, minc=2)
    for t, x in zip(T, X):
        avg.update(x, t)
    dt = np.diff(np.concatenate([[0.0], T]))
    mean = np.tensordot(dt, X, axes=1) / T[-1]
    sd = np.sqrt(np.tensordot(dt, (X - mean) ** 2, axes=1) / T[-1])
    got_mean, got_sd = avg.result()
    assert np.max(np.abs(got_mean - mean)) <= 1e-13 * np.max(np.abs(mean))
    assert np.max(np.abs(got_sd - sd)) <= 1e-10 * np.max(np.abs(sd))
    p = avg.write("t", str(tmp_path))
    rows = np.loadtxt(p)
    assert rows.shape == (n_m, 11)
    assert np.array_equal(rows[:, 0], 2 * np.arange(n_m))
    assert np.allclose(rows[:, 1:11:2], mean, rtol=1e-7) and np.allclose(rows[:, 2:11:2], sd, rtol=1e-7)


def test_spectra_average_of_oracle_run():
    """Snapshot spectra of an oracle run averaged over its log steps; the first
    call sets the mean (n_calls = 1) and the SD starts at zero."""
    from tests.helpers import oracle, seeded
    spec = dict(n_r_max=17, n_cheb_max=17, m_max=8, ek=1e-3, ra=1e5, pr=1.0, radratio=0.35, l_ek_pump=True,
                time_scheme="CNAB2", dtMax=1e-4, matrix_solve="INFLUENCE")
    sim = oracle(spec, temp0=seeded(spec, 1, 1e-2))
    avg = pizza_io.SpectraAverage(sim.M)
    t_avg, snaps, dts = 0.0, [], []
    for k in range(6):
        t_avg += sim.tscheme.dt[0] if hasattr(sim, "tscheme") else 1e-4
        sp = sim.spectra()
        avg.update(sp, t_avg)
        snaps.append(sp)
        dts.append(t_avg - (sum(dts) if dts else 0.0))
        sim.advance()
    mean, sd = avg.result()
    w = np.array(dts)
    ref = np.tensordot(w, np.array(snaps), axes=1) / t_avg
    assert np.max(np.abs(mean - ref)) <= 1e-13 * np.max(np.abs(ref))
    assert np.all(sd >= 0.0) and np.all(np.isfinite(sd))


def test_2d_spectra_match_reference_reader_fixture(tmp_path):
    """The 2D_spec_avg writer against the golden file that the reference's
    own reader parsed (tests/golden/make_2d_spectra_golden.py): the same
    bytes, the same parsed values; and the averages against their closed
    form (getMSD2's recursion)."""
    import json
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_2d_spectra_golden import sample, write_sample
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    p = write_sample(str(tmp_path / "spec2d.bin"))
    with open(p, "rb") as a, open(os.path.join(here, "spec2d_sample.bin"), "rb") as b:
        assert a.read() == b.read()
    with open(os.path.join(here, "spec2d_sample.json")) as f:
        ref = json.load(f)
    got = pizza_io.read_2d_spectra(p)
    for k in ("version", "n_r_max", "n_m_max", "m_max", "minc"):
        assert got[k] == ref[k]
    assert np.array_equal(got["r"], np.array(ref["radius"]))
    for name, key in (("us2", "us2_m"), ("us2_SD", "us2_m_SD"), ("up2", "up2_m"), ("up2_SD", "up2_m_SD"),
                      ("enst", "enst_m")):
        assert np.array_equal(got[name], np.array(ref[key])), name
    cfg, r, snaps, times = sample()
    dts = np.diff((0.0,) + tuple(times))
    mean = sum(d * x for d, x in zip(dts, snaps)) / times[-1]
    var = sum(d * (x - mean) ** 2 for d, x in zip(dts, snaps)) / times[-1]
    np.testing.assert_allclose(got["us2"], mean[0].T, rtol=1e-13)
    np.testing.assert_allclose(got["up2_SD"], np.sqrt(var[1]).T, rtol=1e-10)


def test_force_balance_files_match_reference_reader_fixture(tmp_path):
    """The vort_bal / vort_terms_avg / vphi_bal / vphi_power writers against
    the golden files that the reference's own readers parsed
    (tests/golden/make_balance_golden.py): the same bytes; the parsed
    averages against their closed form (getMSD2's recursion, cc2real r
    height), and the u_phi records as written."""
    import json
    import sys
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, here)
    from make_balance_golden import TERMS, sample, write_sample
    paths = write_sample(str(tmp_path))
    for p in paths:
        with open(p, "rb") as a, open(os.path.join(here, os.path.basename(p)), "rb") as b:
            assert a.read() == b.read(), os.path.basename(p)
    with open(os.path.join(here, "balance_golden.json")) as f:
        ref = json.load(f)
    cfg, r, height, calls = sample()
    assert ref["version"] == 2 and ref["n_r_max"] == len(r) and ref["n_m_max"] == cfg.m_max + 1
    m = np.arange(cfg.m_max + 1)[:, None]

    def cc2(z):
        out = 2.0 * np.abs(z) ** 2
        out[0] = z[0].real ** 2
        return out * r * height
    # equal averaging steps: the mean is the plain mean over the calls
    for key, q in (("buo_mean", "buo"), ("cor_mean", "cor"), ("adv_mean", "adv"), ("domdt_mean", "dwdt"),
                   ("visc_mean", "visc"), ("pump_mean", "pump")):
        want = sum(cc2(c[1][q]) for c in calls) / len(calls)
        np.testing.assert_allclose(np.array(ref[key]), want, rtol=1e-12, err_msg=key)
    want = sum(cc2(c[1]["buo"] + c[1]["cor"]) for c in calls) / len(calls)
    np.testing.assert_allclose(np.array(ref["thwind_mean"]), want, rtol=1e-12)
    v = ref["vphi"]
    assert v["time"] == [c[0] for c in calls]
    np.testing.assert_array_equal(np.array(v["vp"]), np.array([c[2] for c in calls]))
    np.testing.assert_array_equal(np.array(v["rey_stress"]), np.array([c[3]["rey_stress"] for c in calls]))
    np.testing.assert_array_equal(np.array(v["visc"]), np.array([c[3]["visc"] for c in calls]))
    lines = open(paths[3]).read().splitlines()
    assert len(lines) == 3 and all(len(ln) == 20 + 5 * 16 for ln in lines)
    assert TERMS == ("buo", "cor", "adv", "dwdt", "visc", "pump")
