"""The product's host scene builder against the oracle's restatement of the
reference's scene rules (domains, automatic PML, neighbours, update flags,
PML profiles), on the CPU through pstd_scene_build."""
import ctypes

import numpy as np
import pytest

from openpstd_gb300 import _lib, scenes
from openpstd_gb300 import config as C
from openpstd_gb300.config import CConfig, c_domain_info


class HostScene:
    def __init__(self, conf):
        self.cc = CConfig(conf)
        self.h = ctypes.c_void_p()
        _lib.check(_lib.lib().pstd_scene_build(ctypes.byref(self.cc.c), ctypes.byref(self.h)))

    def __del__(self):
        _lib.lib().pstd_destroy(self.h)

    def count(self):
        n = ctypes.c_int32()
        _lib.check(_lib.lib().pstd_scene_domain_count(self.h, ctypes.byref(n)))
        return n.value

    def info(self, i):
        d = c_domain_info()
        _lib.check(_lib.lib().pstd_scene_domain_info(self.h, i, ctypes.byref(d)))
        return d.as_dict()

    def neighbours(self, i, k):
        buf, n = (ctypes.c_int32 * 256)(), ctypes.c_int32()
        _lib.check(_lib.lib().pstd_scene_neighbours(self.h, i, k, buf, 256, ctypes.byref(n)))
        return [buf[j] for j in range(n.value)]

    def attenuation(self, i):
        nx, ny = self.info(i)["size"]
        arrs = [np.zeros(nx, np.float32), np.zeros(nx + 1, np.float32), np.zeros(ny, np.float32),
                np.zeros(ny + 1, np.float32)]
        P = ctypes.POINTER(ctypes.c_float)
        _lib.check(_lib.lib().pstd_scene_attenuation(self.h, i, *[a.ctypes.data_as(P) for a in arrs]))
        return arrs


def _domain_test_conf():
    conf = C.PSTDConfiguration.CreateDefaultConf()
    conf.Domains = [C.DomainConf((0, 0), (50, 60), T=C.DomainConfEdge(0, False), L=C.DomainConfEdge(0.35, True),
                                 B=C.DomainConfEdge(0.25, False), R=C.DomainConfEdge(0.7, False))]
    conf.Speakers, conf.Receivers = [(4.1, 5.1, 0)], []
    return conf


def _default_conf():
    conf = C.PSTDConfiguration.CreateDefaultConf()
    conf.Receivers = []
    return conf


CONFS = {
    "square_200": lambda: scenes.plain_square(0),
    "lshape_full": lambda: scenes.l_shape(0, steps=4000),
    "lshape_seed1": lambda: scenes.l_shape(1, scale=0.25, steps=100),
    "lshape_seed2": lambda: scenes.l_shape(2, scale=0.3, steps=100),
    "domain_test": _domain_test_conf,
    "batch": lambda: scenes.batch_scenes(5, n=1, steps=10)[0],
    "batch2": lambda: scenes.batch_scenes(11, n=1, steps=10)[0],
}


@pytest.mark.parametrize("name", sorted(CONFS))
def test_scene_matches_oracle(oracle_mod, pstd_lib, name):
    conf = CONFS[name]()
    o = oracle_mod.OracleScene(conf, 32)
    p = HostScene(conf)
    assert p.count() == o.n_domains
    for i in range(o.n_domains):
        a, b = p.info(i), o.domain_info(i)
        for key in a:
            if isinstance(a[key], float):
                assert a[key] == pytest.approx(b[key], rel=1e-6), (i, key)
            else:
                assert a[key] == b[key], (i, key)
        for k in range(4):
            assert p.neighbours(i, k) == o.neighbours(i, k), (i, k)
        if b["is_pml"]:
            ax_p, ax_v, ay_p, ay_v = p.attenuation(i)
            np.testing.assert_allclose(o.snapshot(i, "pml_px"), np.broadcast_to(ax_p[None, :], o.field_shape(i, "px")), rtol=2e-6, atol=1e-12)
            np.testing.assert_allclose(o.snapshot(i, "pml_vx"), np.broadcast_to(ax_v[None, :], o.field_shape(i, "vx")), rtol=2e-6, atol=1e-12)
            np.testing.assert_allclose(o.snapshot(i, "pml_py"), np.broadcast_to(ay_p[:, None], o.field_shape(i, "py")), rtol=2e-6, atol=1e-12)
            np.testing.assert_allclose(o.snapshot(i, "pml_vy"), np.broadcast_to(ay_v[:, None], o.field_shape(i, "vy")), rtol=2e-6, atol=1e-12)


def test_default_configuration_scene(oracle_mod, pstd_lib):
    # CreateDefaultConf: two domains with an offset shared edge (partly covered edges)
    conf = _default_conf()
    try:
        o = oracle_mod.OracleScene(conf, 32)
    except oracle_mod.OracleError as e:
        assert e.code == _lib.PSTD_ERR_UNSUPPORTED
        with pytest.raises(_lib.PSTDError) as pe:
            HostScene(conf)
        assert pe.value.code == _lib.PSTD_ERR_UNSUPPORTED
        return
    p = HostScene(conf)
    assert p.count() == o.n_domains


def _rejects_both(oracle_mod, conf, code):
    with pytest.raises(oracle_mod.OracleError) as oe:
        oracle_mod.OracleScene(conf, 32)
    assert oe.value.code == code
    with pytest.raises(_lib.PSTDError) as pe:
        HostScene(conf)
    assert pe.value.code == code


def test_rejects_two_vacant_runs(oracle_mod, pstd_lib):
    # a neighbour in the middle of an edge leaves two uncovered runs, which the
    # reference's vacant-range table cannot represent
    conf = scenes.plain_square(0, n=200, steps=10)
    dx = 0.2
    conf.Domains.append(scenes._domain(200, 80, 60, 40, dx, dict(left=1.0, right=1.0, top=1.0, bottom=1.0)))
    _rejects_both(oracle_mod, conf, _lib.PSTD_ERR_UNSUPPORTED)


def test_rejects_power_of_two_transform(oracle_mod, pstd_lib):
    # N + 2W = 128 makes the transform and derivative-factor lengths disagree
    conf = scenes.plain_square(0, n=64, steps=10)
    with pytest.raises(_lib.PSTDError) as pe:
        HostScene(conf)
    assert pe.value.code == _lib.PSTD_ERR_UNSUPPORTED
    s = oracle_mod.OracleScene(conf, 32)   # the oracle notices when it computes
    with pytest.raises(oracle_mod.OracleError) as oe:
        s.run(1)
    assert oe.value.code == _lib.PSTD_ERR_UNSUPPORTED


def test_rejects_transposed_receiver(oracle_mod, pstd_lib):
    # receivers read p0(x offset, y offset): x offset must be < Ny
    conf = scenes.l_shape(0, scale=0.2, steps=10)
    conf.Receivers = [(40.0, 10.0, 0.0)]   # x offset 200 cells in a 240x120 domain
    _rejects_both(oracle_mod, conf, _lib.PSTD_ERR_UNSUPPORTED)


def test_rejects_window_wider_than_pml(oracle_mod, pstd_lib):
    conf = scenes.plain_square(0, n=60, steps=10, pml=20)
    with pytest.raises(_lib.PSTDError) as pe:
        HostScene(conf)
    assert pe.value.code == _lib.PSTD_ERR_UNSUPPORTED
    s = oracle_mod.OracleScene(conf, 32)   # the oracle notices only when it computes
    with pytest.raises(oracle_mod.OracleError):
        s.run(1)
