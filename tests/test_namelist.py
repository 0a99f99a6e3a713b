"""input.nml reading (pizza_gb300.namelist) and the start field of the GPU
driver (pizza_gb300.run); no GPU needed."""
import numpy as np

from pizza_gb300 import namelist, pizza_io
from pizza_gb300.run import start_temperature

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
    ts = start_temperature(cfg, ctl, seed=7)
    assert np.count_nonzero(ts[0]) == 0 and np.all(np.abs(ts[1:, 1:-1]) > 0)
