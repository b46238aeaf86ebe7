"""The C host front end against the reference's regrid output (golden
fixtures): mesh coordinates and homogenized conductivities bit for bit."""
import numpy as np
import pytest

from libemmi_mgfd_gb300 import host
from libemmi_mgfd_gb300 import workloads as W

CASES = {
    "tiny_layered": lambda: W.tiny_layered(),
    "tiny_aniso": lambda: W.tiny_aniso(n=(16, 8, 16)),
    "c1_layered_64": lambda: W.config1(64),
}


@pytest.fixture(scope="module", autouse=True)
def _built():
    from libemmi_mgfd_gb300 import build
    build.build()


@pytest.mark.parametrize("name", sorted(CASES))
def test_regrid_bitwise(golden, name):
    g = golden(name)
    s = CASES[name]()
    m = host.Model.from_survey(s)
    src = g["srcrec"][:3]
    out = m.regrid(*[float(v) for v in src])
    for nm in host.GRID_FIELDS:
        assert np.array_equal(out[nm], g[nm]), nm
    assert m.rho_water() == float(g["rho_water"][0])


def test_create_nugrid_uniform_and_stretched():
    import ctypes as C
    L = host.lib()
    x = np.zeros(11, np.float32)
    r = L.eh_create_nugrid(10, C.c_float(500.0), C.c_float(100.0), x.ctypes.data_as(C.c_void_p))
    assert r == 1.0 and np.allclose(x, np.arange(11) * 100.0)
    r = L.eh_create_nugrid(10, C.c_float(5e4), C.c_float(100.0), x.ctypes.data_as(C.c_void_p))
    assert r > 1.0 and abs(x[-1] - 5e4) / 5e4 < 1e-5
    assert np.all(np.diff(x) > 0)


def test_search_past_padded_axis_is_reported():
    s = W.tiny_layered()
    m = host.Model.from_survey(s)
    m.nx = 200  # the reference sizes its source-depth search by nx
    m.rho11 = np.ones((s.nz, s.ny, 200), np.float32)
    m.rho22 = m.rho11
    m.rho33 = m.rho11
    with pytest.raises(RuntimeError):
        m.regrid(0.0, 0.0, 2100.0)


def test_batched_vti_mesh_axes_match_reference(golden):
    """The 25-shot VTI/bathymetry configuration on the 48x48x64 mesh its
    reference fixture was made on: both fixture shots' mesh axes bit for
    bit (the reference's own run, tests/golden/c2_vti_48x48x64_ref.npz)."""
    g = golden("c2_vti_48x48x64_ref")
    s = W.config2(96)
    s.n = tuple(int(v) for v in g["n"])
    m = host.Model.from_survey(s)
    xx, yy, zz, _ = m.padded()
    for k in g["shots"]:
        src = s.sources[int(k) - 1]
        ax = m.axes(xx, yy, zz, float(src[0]), float(src[1]), float(src[2]))
        for nm in ("x1", "x2", "x3"):
            assert np.array_equal(ax[nm], g[f"s{k}_{nm}"]), (k, nm)


def test_mesh_without_a_geometric_ratio_is_reported():
    """The same configuration on a 40^3 mesh: the source lies 39 padded
    cells down, one cell is left for the bottom stretch, and the
    reference's fixed-point loop for its ratio never ends
    (src/create_nugrid.c:24-31).  The front end reports EH_ENUGRID."""
    import ctypes as C
    s = W.config2(40)
    m = host.Model.from_survey(s)
    xx, yy, zz, _ = m.padded()
    src = s.sources[0]
    with pytest.raises(RuntimeError, match=r"\(-3\)"):
        m.axes(xx, yy, zz, float(src[0]), float(src[1]), float(src[2]))
    x = np.zeros(2, np.float32)
    r = host.lib().eh_create_nugrid(1, C.c_float(5e4), C.c_float(20.0),
                                    x.ctypes.data_as(C.c_void_p))
    assert r == 0.0
