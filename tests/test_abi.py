"""C ABI checks that need no GPU: the library loads, exports every entry
point declared in include/pizza_gpu.h, and the configuration mirror matches."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pizza_gpu.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pz_[a-z_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from pizza_gb300 import build as b
    b.build()
    import pizza_gb300 as pz
    return pz.load_library()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("pz_create", "pz_set_state", "pz_step", "pz_get_state", "pz_get_series", "pz_destroy",
              "pz_last_error", "pz_config_default"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_config_default_matches_reference_namelist_defaults(lib):
    import pizza_gb300 as pz
    c = pz._CConfig()
    lib.pz_config_default(ctypes.byref(c))
    # src/namelists.f90:530-672
    assert (c.n_r_max, c.m_max, c.minc) == (32, 32, 1)
    assert (c.ra, c.ek, c.pr, c.radratio) == (1.0e5, 1.0e-3, 1.0, 0.35)
    assert (c.ktopt, c.kbott, c.ktopv, c.kbotv) == (1, 1, 2, 2)
    assert (c.dtMax, c.courfac, c.alpha, c.dt_fac) == (1.0e-5, 1.0e3, 0.5, 2.0)
    assert c.matrix_solve == pz.SOLVE_DIRECT and c.buo_imp == 1 and c.corio_imp == 1


def test_python_config_mirror_round_trip():
    import pizza_gb300 as pz
    cfg = pz.Config(n_r_max=33, m_max=32, time_scheme="SBDF3", matrix_solve="influence", l_ek_pump=True)
    c = cfg.to_c()
    assert c.n_cheb_max == 33 and c.time_scheme == pz.SCHEMES["SBDF3"]
    assert c.matrix_solve == pz.SOLVE_INFLUENCE and c.l_ek_pump == 1
    assert cfg.n_m_max == 33 and cfg.n_phi_max == 96
    with pytest.raises(ValueError):
        pz.Config(time_scheme="RK4").to_c()
