"""The CPU oracle against the known answers of openPSTD's own unit tests.

Every expected value comes from tests/golden/reference_kats.json, which
tests/golden/make_golden.py extracts from the reference's test/Kernel/*.cpp.
Tolerances follow the reference checks: Eigen isApprox (relative 1e-5 for
float) and is_approx (EPSILON = 1e-5, kernel/core/kernel_functions.cpp:341-350).
"""
import numpy as np
import pytest

from openpstd_gb300 import config as C

f32 = np.float32


def is_approx(a, b, eps=1e-5):
    """kernel/core/kernel_functions.cpp:341-350."""
    return abs(b) < eps if a == 0 else abs((a - b) / a) < eps


def eigen_is_approx(x, y, prec=1e-5):
    x, y = np.asarray(x, float), np.asarray(y, float)
    return np.linalg.norm(x - y) <= prec * min(np.linalg.norm(x), np.linalg.norm(y))


def linspaced(lo, hi, n):
    """Eigen LinSpaced in float: low + i * ((high - low) / (n - 1))."""
    lo, hi = f32(lo), f32(hi)
    step = f32((hi - lo) / f32(n - 1))
    return (lo + np.arange(n, dtype=f32) * step).astype(f32)


def test_next_2_power(oracle_mod, golden):
    for n, want in golden["next_2_power"]:
        assert oracle_mod.next_2_power(n) == want


def test_window_size(oracle_mod):
    # patch error 70 -> 32 (kernel/KernelInterface.cpp:128-134)
    assert oracle_mod.window_size(70) == 32
    s = C.PSTDSettings()
    s.SetPatchError(70)
    assert s.GetWindowSize() == 32


@pytest.mark.parametrize("case", ["rho_array_one_neighbour", "rho_array_two_neighbour"])
def test_rho_arrays(oracle_mod, golden, case):
    g = golden[case]
    p, v = oracle_mod.rho_array(*g["rho"])
    assert eigen_is_approx(p.ravel(), g["pressure"])
    assert eigen_is_approx(v.ravel(), g["velocity"]) or np.allclose(v.ravel(), g["velocity"], atol=1e-9)


def test_window_generator(oracle_mod, golden):
    g = golden["window_generator"]
    w = oracle_mod.window(g["W"], g["patch_error"])
    assert eigen_is_approx(w, g["values"])
    assert len(w) == 2 * g["W"] + 1


def test_wisdom_cache_values(oracle_mod, golden):
    g = golden["wisdom_cache"]
    d = oracle_mod.discretization(g["dx"], g["N"])
    assert len(d["wave_numbers"]) == 128        # 2^ceil(log2 115)
    for field, part, i, want in g["checks"]:
        if field == "wave_numbers":
            got = d["wave_numbers"][i]
        elif field == "complex_factors":
            got = d["complex_imag"][i] if part == "imag" else 0.0
        else:
            arr = d["pressure"] if field.startswith("pressure") else d["velocity"]
            got = arr[i].real if part == "real" else arr[i].imag
        assert is_approx(want, got), (field, part, i, want, got)


def test_wisdom_cache_matching(oracle_mod):
    # test/Kernel/WisdomCache.cpp:48-64: 178 and 227 share a length, twice that of 115
    a, b, c = (len(oracle_mod.discretization(0.2, n)["wave_numbers"]) for n in (115, 178, 227))
    assert b == c == 2 * a
    k = oracle_mod.discretization(0.2, 115)["wave_numbers"]
    assert k.max() <= 15.8 and k.min() >= 0


def test_derivative_factors_match_listed_table(oracle_mod, golden):
    # the 128-entry pressure/velocity tables listed in test_spatderp3 (dx = 0.4);
    # only bins 0..L/2 enter the transform
    # (the listed table was computed in double precision)
    g = golden["spatderp3"]
    n = 65
    for prec, rtol, atol in ((64, 1e-7, 1e-7), (32, 0, 8e-6 * 7.9)):
        d = oracle_mod.discretization(g["dx"], g["N"], prec)
        assert np.allclose(d["pressure"].real[:n], g["real_p"][:n], rtol=rtol, atol=atol)
        assert np.allclose(d["pressure"].imag[:n - 1], g["imag_p"][:n - 1], rtol=rtol, atol=atol)
        assert np.allclose(d["velocity"].real[:n], g["real_v"][:n], rtol=rtol, atol=atol)
        assert np.allclose(d["velocity"].imag[:n - 1], g["imag_v"][:n - 1], rtol=rtol, atol=atol)
        # the Nyquist entry is real up to the rounding of cos(pi/2)
        assert abs(d["pressure"].imag[n - 1]) < 1e-5


@pytest.mark.parametrize("precision", [32, 64])
def test_spatderp3_sin_to_cos(oracle_mod, golden, precision):
    """test/Kernel/kernel_functions.cpp:92-143: sin on the staggered grid -> cos."""
    g = golden["spatderp3"]
    ls = {k: linspaced(*v) for k, v in g["linspace"].items()}
    d = oracle_mod.discretization(g["dx"], g["N"], precision)
    w = np.array(g["window"])
    rp = oracle_mod.spatderp3(np.sin(ls["d1p"]), np.sin(ls["d2p"]), np.sin(ls["d3p"]), d["pressure"], w,
                              g["wlen"], 1.2, 1.2, 1.2, velocity=False, precision=precision)
    rv = oracle_mod.spatderp3(np.sin(ls["d1v"]), np.sin(ls["d2v"]), np.sin(ls["d3v"]), d["velocity"], w,
                              g["wlen"], 1.2, 1.2, 1.2, velocity=True, precision=precision)
    assert len(rp) == 51 and len(rv) == 50
    assert eigen_is_approx(np.cos(ls["d2v"]), rp)
    assert eigen_is_approx(np.cos(ls["d2p"]), rv)


def _domain_test_conf():
    """create_a_scene of test/Kernel/Domain.cpp:47-71."""
    conf = C.PSTDConfiguration.CreateDefaultConf()
    d = C.DomainConf((0, 0), (50, 60), T=C.DomainConfEdge(0, False), L=C.DomainConfEdge(0.35, True),
                     B=C.DomainConfEdge(0.25, False), R=C.DomainConfEdge(0.7, False))
    conf.Settings.SetGridSpacing(0.2)
    conf.Domains = [d]
    conf.Speakers = [(4.1, 5.1, 0)]
    conf.Receivers = []
    return conf


def test_speaker_initial_values(oracle_mod, golden):
    g = golden["speaker_initial_values"]
    s = oracle_mod.OracleScene(_domain_test_conf())
    p0 = s.snapshot(0, "p0")
    assert p0[25, 20] == g["p0_25_20"]
    assert p0[24, 20] == p0[25, 21]
    assert is_approx(p0[24, 20], g["p0_24_20"])


def test_domain_scene_from_config(oracle_mod, golden):
    g = golden["domain_scene"]
    s = oracle_mod.OracleScene(_domain_test_conf())
    assert s.n_domains == g["n_domains"]
    air = s.domain_info(0)
    assert air["top_left"][0] == 0 and air["size"][0] == g["size_x"]
    assert air["top_left"][1] + air["size"][1] == g["bottom_right_y"]
    assert sum(air["n_neighbours"]) == g["air_neighbours_with_pml"]
    for i in range(1, s.n_domains):
        assert s.domain_info(i)["is_pml"]


def test_scene_pml_creation(oracle_mod, golden):
    """test/Kernel/Scene.cpp:48-123."""
    g = golden["scene_pml"]
    conf = C.PSTDConfiguration.CreateDefaultConf()
    conf.Domains = [C.DomainConf((0, 0), tuple(g["size_world"]), *(C.DomainConfEdge(g["alpha"], False) for _ in range(4)))]
    conf.Speakers = [(4.1, 5.1, 0)]
    conf.Receivers = []
    conf.Settings.SetPMLCells(g["pml_cells"])
    s = oracle_mod.OracleScene(conf)
    infos = [s.domain_info(i) for i in range(s.n_domains)]
    assert len(infos) == g["n_domains"]
    assert sum(i["is_pml"] for i in infos) == g["n_pml"]
    assert sum(i["is_secondary_pml"] for i in infos) == g["n_secondary"]
    for i in infos:
        if i["is_pml"]:
            assert g["pml_cells"] in i["size"]
        if i["is_secondary_pml"]:
            assert i["size"] == (g["pml_cells"], g["pml_cells"])
