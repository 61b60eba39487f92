"""Host-side API behaviour of the GB300 package (no GPU needed).

These mirror the reference's own API tests (tests/test_grid.py:17-44,
tests/test_sources.py:17-43, tests/test_boundaries.py:19-77,
tests/test_backend.py:22-26) plus the registration rules the fused kernels
rely on.  Nothing here runs a time step.
"""

import os

import numpy as np
import pytest
import torch

import golden_scenes
from oracle import fdtd_oracle as fo


@pytest.fixture
def grid(fd):
    return fd.Grid(shape=(10, 10, 10), grid_spacing=100e-9, permittivity=1.0, permeability=1.0)


def test_grid_shape(fd):
    assert fd.Grid(shape=(3, 3, 3)).shape == (3, 3, 3)
    assert fd.Grid(shape=(10.0e-9, 10.0e-9, 10.0e-9), grid_spacing=5.0e-9).shape == (2, 2, 2)
    assert fd.Grid(shape=(10.0e-9, 10.0e-9, 3), grid_spacing=5.0e-9).shape == (2, 2, 3)


@pytest.mark.parametrize("shape,expect", [((3, 1, 1), 1.0), ((3, 3, 1), 0.5 ** 0.5), ((3, 3, 3), (1 / 3) ** 0.5)])
def test_default_courant(fd, shape, expect):
    g = fd.Grid(shape=shape)
    assert g.courant_number == pytest.approx(expect, rel=0.02)
    assert g.courant_number == 0.99 * expect or g.courant_number == pytest.approx(0.99 * expect, rel=1e-15)


def test_courant_too_high(fd):
    with pytest.raises(ValueError):
        fd.Grid(shape=(3, 3, 3), courant_number=0.6)


def test_set_backend_names(fd):
    assert fd.set_backend("gb300.float32").float == torch.float32
    assert fd.backend.precision == "float32"
    assert fd.set_backend("gb300.float32c").compensated
    assert fd.set_backend("gb300").float == torch.float64
    assert fd.set_backend("gb300.cuda.float32").precision == "float32"
    for bad in ("numpy", "torch.float32", "torch.cuda", "gb300.float16", "foo", "gb300.cpu.float32"):
        with pytest.raises(ValueError):
            fd.set_backend(bad)


def test_grid_dtype_follows_backend(fd):
    fd.set_backend("gb300.float32")
    g = fd.Grid((4, 4, 4))
    assert g.E.dtype == torch.float32 and g.inverse_permittivity.dtype == torch.float32
    fd.set_backend("gb300.float32c")
    g = fd.Grid((4, 4, 4))
    assert g._E_lo is not None and g._E_lo.shape == (4, 4, 4, 3)
    fd.set_backend("gb300.float64")
    g = fd.Grid((4, 4, 4), permittivity=np.full((4, 4, 4), 2.0))
    assert g.inverse_permittivity.dtype == torch.float64
    assert torch.all(g.inverse_permittivity.cpu() == 0.5)


def test_plane_source_polarization_error(grid, fd):
    with pytest.raises(ValueError):
        grid[0, :, :] = fd.PlaneSource(polarization="x")
    with pytest.raises(ValueError):
        grid[:, 0, :] = fd.PlaneSource(polarization="y")
    with pytest.raises(ValueError):
        grid[:, :, 0] = fd.PlaneSource(polarization="z")
    assert grid.sources == []  # a rejected source is not left half-registered


@pytest.mark.parametrize("key,pol,epol,hpol", [
    ((0, slice(None), slice(None)), "y", 1, 2), ((0, slice(None), slice(None)), "z", 2, 1),
    ((slice(None), 0, slice(None)), "x", 0, 2), ((slice(None), 0, slice(None)), "z", 2, 0),
    ((slice(None), slice(None), 0), "x", 0, 1), ((slice(None), slice(None), 0), "y", 1, 0)])
def test_plane_source_polarization_inference(grid, fd, key, pol, epol, hpol):
    ps = fd.PlaneSource(polarization=pol)
    grid[key] = ps
    assert ps._Epol == epol and ps._Hpol == hpol


def test_plane_source_not_a_plane(grid, fd):
    with pytest.raises(ValueError):
        grid[0:3, 0:3, 0:3] = fd.PlaneSource(polarization="x")
    with pytest.raises(ValueError):
        grid[0, 0, :] = fd.PlaneSource(polarization="z")


def test_periodic_boundary(grid, fd):
    pb = fd.PeriodicBoundary(name="periodic_boundary")
    grid[0, :, :] = pb
    assert pb in grid.boundaries and pb.axis == 0
    with pytest.raises(IndexError):
        fd.Grid((10, 10, 10))[0:2, :, :] = fd.PeriodicBoundary()
    with pytest.raises(IndexError):
        fd.Grid((10, 10, 10))[2, :, :] = fd.PeriodicBoundary()
    with pytest.raises(AttributeError):
        grid[-1, :, :] = fd.PeriodicBoundary()


def test_pml_placement(grid, fd):
    pml = fd.PML(name="PML")
    grid[0:3, :, :] = pml
    assert pml in grid.boundaries and (pml.axis, pml.high, pml.thickness) == (0, 0, 3)
    with pytest.raises(IndexError):
        fd.Grid((10, 10, 10))[2:4, :, :] = fd.PML()
    with pytest.raises(ValueError):
        fd.Grid((10, 10, 10))[[0, 1], :, :] = fd.PML()
    with pytest.raises(AttributeError):
        grid[0:2, :, :] = fd.PML()
    p = fd.PML()
    grid[:, -4:, :] = p
    assert (p.axis, p.high, p.thickness, p.start) == (1, 1, 4, 6)
    assert p.psi_E.shape == (10, 4, 10, 2)


def test_domain_border_pml(grid, fd):
    with pytest.raises(IndexError):
        fd.DomainBorderPML(grid, grid.Nx // 2 + 1)
    fd.DomainBorderPML(grid, 3)
    assert sorted((b.axis, b.high) for b in grid.boundaries) == [(a, h) for a in range(3) for h in range(2)]


def test_duplicate_names(grid, fd):
    grid[0:2, :, :] = fd.PML(name="dup")
    with pytest.raises(ValueError):
        grid[3, 3, 3] = fd.PointSource(name="dup")


def test_point_and_line_source_registration(grid, fd):
    with pytest.raises(ValueError):
        grid[1:3, 1, 1] = fd.PointSource()
    with pytest.raises(ValueError):
        grid[1, 1, 1:2] = fd.LineSource()
    src = fd.PointSource(period=155e-9 * 10 / 299792458.0)
    grid[4, 4, 4] = src
    assert isinstance(src.period, int) and src.period > 0


@pytest.mark.parametrize("name", sorted(golden_scenes.SCENES))
def test_registration_matches_oracle(fd, name):
    """Coefficients, object arrays, source profiles and detector points of the
    GB300 host side equal the oracle's for every golden scene."""
    fd.set_backend("gb300.float64")
    g, _, _ = golden_scenes.SCENES[name](fd)
    o, _, _ = golden_scenes.SCENES[name](fo)
    assert g.courant_number == o.courant_number and g.time_step == o.time_step
    assert np.array_equal(g.inverse_permittivity.cpu().numpy(), o.inverse_permittivity)
    assert np.array_equal(g.inverse_permeability.cpu().numpy(), o.inverse_permeability)
    pmls = [b for b in g.boundaries if isinstance(b, fd.PML)]
    opmls = [b for b in o.boundaries if isinstance(b, fo.PML)]
    assert len(pmls) == len(opmls)
    for b, ob in zip(pmls, opmls):
        assert (b.axis, b.high, b.thickness) == (ob.axis, ob.high, ob.thickness)
        for name_ in ("bE", "cE", "bH", "cH"):
            assert np.array_equal(getattr(b, name_[0].lower() + "_" + name_[1]).cpu().numpy(), getattr(ob, name_))
    for obj, oobj in zip(g.objects, o.objects):
        assert np.array_equal(obj.inverse_permittivity.cpu().numpy(), oobj.inverse_permittivity)
        if hasattr(oobj, "absorption_factor"):
            assert np.array_equal(obj.absorption_factor.cpu().numpy(), oobj.absorption_factor)
    for s, os_ in zip(g.sources, o.sources):
        if isinstance(s, fd.SoftArbitraryPointSource):
            assert (s.x, s.y, s.z, s.impedance) == (os_.x, os_.y, os_.z, os_.impedance)
            for q in (0, 3, 59, 60, 100):
                vin = os_.waveform_array[q] if q < os_.waveform_array.shape[0] else 0.0
                assert s._value(q) == vin
            continue
        assert s.period == os_.period
        if isinstance(s, fd.LineSource):
            assert np.array_equal(np.asarray(s.profile), os_.profile)
        scale = os_.amplitude if isinstance(os_, fo.PointSource) else 1.0
        for q in (0, 3, 17, 40):
            assert s._value(q) == scale * os_.wave(q)
    for det, odet in zip(g.detectors, o.detectors):
        assert (list(det.x), list(det.y), list(det.z)) == (list(odet.x), list(odet.y), list(odet.z))


def test_pml_reference_views(fd):
    fd.set_backend("gb300.float64")
    g = fd.Grid((8, 9, 10))
    p = fd.PML()
    g[:, :, 0:4] = p
    assert p.bE.shape == (8, 9, 4, 3) and p.cE[..., 0].abs().max() == 0
    assert torch.allclose(p.cE[0, 0, :, 2].cpu(), p.c_E.cpu())
    assert p.psi_Ex.shape == (8, 9, 4, 3) and p.phi_E.shape == (8, 9, 4, 3)


def test_no_cpu_time_step(fd):
    if torch.cuda.is_available():
        pytest.skip("CUDA present")
    g = fd.Grid((4, 4, 4))
    with pytest.raises(RuntimeError):
        g.run(1)
    with pytest.raises(RuntimeError):
        g.update_E()


def test_unsupported_components(grid, fd):
    with pytest.raises(NotImplementedError):
        fd.Object(permittivity=1 + 1j)


def test_soft_arbitrary_point_source_registration(grid, fd):
    """fdtd/sources.py:562-598: one cell; the source registers its own
    CurrentDetector at the cell (named <name>_I here; the reference raises
    UnboundLocalError for a named source)."""
    with pytest.raises(ValueError):
        grid[4:6, 4, 4] = fd.SoftArbitraryPointSource(np.zeros(4))
    assert not grid.sources
    src = fd.SoftArbitraryPointSource(np.ones(4), impedance=50.0, name="port")
    grid[4, 5, 6] = src
    assert grid.port is src and grid.sources == [src]
    det = src.current_detector
    assert grid.port_I is det and det in grid.detectors
    assert (det.x, det.y, det.z) == ([4], [5], [6]) and det._rec_shape == (1, 1, 1)
    assert (src.x, src.y, src.z) == (4, 5, 6)
    assert src._value(3) == 1.0 and src._value(4) == 0.0
    cd = fd.CurrentDetector(name="loop")
    grid[2:4, 3:5, 7] = cd  # inclusive ranges like BlockDetector
    assert (cd.x, cd.y, cd.z) == ([2, 3, 4], [3, 4, 5], [7]) and not hasattr(cd, "E")
    assert cd.detector_values()["I"] is cd.I


def test_single_point_current_matches_oracle(fd):
    """CurrentDetector.single_point_current (fdtd/detectors.py:404-464) on the
    grid's present H, against the oracle's restatement, including the index
    wrap at the grid's first planes."""
    fd.set_backend("gb300.float64")
    g = fd.Grid((6, 5, 4), grid_spacing=100e-9)
    o = fo.Grid((6, 5, 4), grid_spacing=100e-9)
    det, odet = fd.CurrentDetector(), fo.CurrentDetector()
    g[2, 2, 2] = det
    o[2, 2, 2] = odet
    h = np.random.default_rng(5).standard_normal((6, 5, 4, 3))
    g.H[...] = torch.as_tensor(h, device=g.H.device)
    o.H[...] = h
    for p in [(2, 2, 2), (0, 0, 0), (5, 4, 3), (0, 3, 1)]:
        assert float(det.single_point_current(*p)) == float(odet._point(*p))


def test_components_with_step_hooks_are_refused(grid, fd):
    """The reference's Grid calls update_E/update_H/update_phi_*/detect_*
    hooks of its components every half step; a component that brings such a
    hook (a user subclass) cannot run inside the fused time step, so
    registering it raises NotImplementedError instead of ignoring the hook."""

    class MySource(fd.PointSource):
        def update_E(self):
            pass

    class MyDetector(fd.LineDetector):
        def detect_H(self):
            pass

    with pytest.raises(NotImplementedError):
        grid[4, 4, 4] = MySource(period=10)
    with pytest.raises(NotImplementedError):
        grid[:, 4, 4] = MyDetector()
    assert grid.sources == [] and grid.detectors == []
    grid[4, 4, 4] = fd.PointSource(period=10)  # the package's own components carry no hooks


def test_plotting_and_complex_raise(grid):
    """Plotting (fdtd/visualization.py) and complex fields are outside this
    backend: the reference's method names exist and raise NotImplementedError."""
    for call in (grid.visualize, grid.generate_video, grid.promote_dtypes_to_complex):
        with pytest.raises(NotImplementedError):
            call()


def test_plotting_helpers_raise(fd):
    for fn in (fd.dB_map_2D, fd.plot_detection, fd.visualization.visualize):
        with pytest.raises(NotImplementedError):
            fn()


def test_curl_functions_need_a_gpu(fd):
    if torch.cuda.is_available():
        pytest.skip("CUDA present")
    with pytest.raises(RuntimeError):
        fd.grid.curl_E(np.zeros((3, 3, 3, 3)))


def test_save_data_keys_without_steps(fd, tmp_path, monkeypatch):
    """Grid.save_data before any step: both '(E)' and '(H)' keys for every
    E/H detector (fdtd/grid.py:508-513), empty record arrays; a DFT plane
    detector stores its accumulators."""
    monkeypatch.chdir(tmp_path)
    g = fd.Grid((10, 9, 8), grid_spacing=155e-9)
    g[:, 4, 4] = fd.LineDetector(name="line")
    g[2:4, 2:4, 2:4] = fd.BlockDetector(name="block")
    g[:, :, 5] = fd.DFTPlaneDetector(frequencies=[1e14], name="dft")
    with pytest.raises(Exception):
        g.save_data()  # no folder yet, as in the reference
    folder = g.save_simulation("keys")
    g.save_data()
    got = np.load(os.path.join(folder, "detector_readings.npz"))
    assert set(got.files) == {"line (E)", "line (H)", "block (E)", "block (H)", "dft (dft)"}
    assert got["line (E)"].shape == (0, 10, 3) and got["block (H)"].shape == (0, 3, 3, 3, 3)
    assert got["dft (dft)"].shape == (1, 10, 9, 1, 3)
