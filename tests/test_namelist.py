"""input.nml reading (pizza_gb300.namelist) and the start field of the GPU
driver (pizza_gb300.run); no GPU needed."""
import numpy as np
import pytest

from oracle.pizza_oracle import Params, Pizza
from pizza_gb300 import namelist, pizza_io
from pizza_gb300.run import run, start_temperature
from pizza_gb300.start_fields import init_prop

NML = """
&grid
 n_r_max    =33,          ! radial points
 n_cheb_max =31,
 m_max      =32,
 minc       =1,
/
&control
 tag        ="case1",
 n_time_steps=200,
 dtMax      =1.0d-4,
 courfac    =2.5D0,
 time_scheme='ARS233',
 l_ek_pump  =.true.,
 matrix_solve='influence',
 runHours   =12,
/
&phys_param
 ra         =1.5E+05,
 ek         =1.0d-3,
 pr         =1.0d0,
 radratio   =0.35d0,
 ktopv      =2, kbotv=2,
/
&start_field
 init_t     =3,
 amp_t      =2.5d-4,
/
&output_control
 n_log_step =10,
 l_2D_spectra = F,
/
"""


def test_parse_groups_values_and_comments(tmp_path):
    g = namelist.parse(NML)
    assert set(g) == {"grid", "control", "phys_param", "start_field", "output_control"}
    assert g["grid"]["n_r_max"] == 33 and g["control"]["dtmax"] == 1.0e-4
    assert g["control"]["courfac"] == 2.5 and g["phys_param"]["ra"] == 1.5e5
    assert g["control"]["l_ek_pump"] is True and g["output_control"]["l_2d_spectra"] is False
    assert g["control"]["time_scheme"] == "ARS233" and g["control"]["tag"] == "case1"
    assert g["phys_param"]["kbotv"] == 2


def test_read_maps_config_controls_and_ignored(tmp_path):
    p = tmp_path / "input.nml"
    p.write_text(NML)
    cfg, ctl, ignored = namelist.read(str(p))
    assert (cfg.n_r_max, cfg.n_cheb_max, cfg.m_max, cfg.minc) == (33, 31, 32, 1)
    assert cfg.dtMax == 1.0e-4 and cfg.courfac == 2.5 and cfg.time_scheme == "ARS233"
    assert cfg.l_ek_pump is True and cfg.matrix_solve == "influence" and cfg.ra == 1.5e5
    assert ctl == {"tag": "case1", "n_time_steps": 200, "init_t": 3, "amp_t": 2.5e-4, "n_log_step": 10,
                   "runhours": 12}
    assert ignored == {"output_control.l_2d_spectra": False}
    cfg.to_c()          # the values convert to the C configuration


def test_start_field_init_t_mode(tmp_path):
    p = tmp_path / "input.nml"
    p.write_text(NML)
    cfg, ctl, _ = namelist.read(str(p))
    t = start_temperature(cfg, ctl)
    r = pizza_io._grid_r(33, 0.35)
    r_i = 0.35 / 0.65
    assert t.shape == (33, 33)
    assert np.allclose(t[3].real, 2.5e-4 * np.sin(np.pi * (r - r_i)), rtol=0, atol=1e-18)
    assert np.count_nonzero(np.delete(t, 3, axis=0)) == 0
    # a seed only replaces pizza's random modes (init_t < -1)
    assert np.array_equal(start_temperature(cfg, ctl, seed=7), t)
    ts = start_temperature(cfg, dict(ctl, init_t=-2), seed=7)
    assert np.count_nonzero(ts[0]) == 0 and np.all(np.abs(ts[1:, 1:-1]) > 0)
    with pytest.raises(ValueError):
        start_temperature(cfg, dict(ctl, init_t=-2))


@pytest.mark.parametrize("init", [-1, 4])
def test_init_prop_matches_oracle(init):
    """initProp's single-mode and bubble starts (init_fields.f90:260-376)
    against the oracle's restatement, on a grid with minc = 1 and 2."""
    for minc in (1, 2):
        spec = dict(n_r_max=33, n_cheb_max=33, m_max=32, minc=minc, ek=1e-3, ra=1e5, radratio=0.35,
                    dtMax=1e-4, matrix_solve="INFLUENCE")
        sim = Pizza(Params(**spec))
        sim.start()
        base = sim.temp.copy()
        sim._init_prop(init, 1e-2)
        want = sim.temp - base
        got = init_prop(33, 32, minc, 0.35, init, 1e-2)
        assert got.shape == want.shape
        assert np.max(np.abs(got - want)) <= 1e-15 * np.max(np.abs(want)), (init, minc)


def test_driver_refuses_options_that_change_the_physics(tmp_path):
    p = tmp_path / "input.nml"
    p.write_text(NML.replace("&start_field", "&start_field\n init_u = 1,"))
    with pytest.raises(ValueError, match="init_u"):
        run(str(p), str(tmp_path))
    p.write_text(NML.replace("&phys_param", "&phys_param\n t_bot = 1.0, 0.5,"))
    with pytest.raises(ValueError, match="t_bot"):
        run(str(p), str(tmp_path))
    p.write_text(NML.replace("&control", "&control\n bc_method = 'galerkin',"))
    with pytest.raises(ValueError, match="bc_method"):
        run(str(p), str(tmp_path))
