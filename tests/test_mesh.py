"""Host-side meshes, contour schedules and wall potentials of the package
(adscf_gb300.mesh) against the oracle's restatement of the reference."""
import numpy as np
import pytest

from adscf_gb300 import mesh
from oracle import film as of
from oracle import interactions as oi


@pytest.mark.parametrize("mtype", [0, 1, 2])
@pytest.mark.parametrize("film3d", [True, False])
@pytest.mark.parametrize("gz", [64, 120, 200])
def test_generate_mesh(mtype, film3d, gz):
    d1, z1 = mesh.generate_mesh(mtype, gz, 3.0, 0.4, film3d=film3d)
    d2, z2 = of.generate_mesh(mtype, gz, 3.0, 0.4, film3d=film3d)
    assert np.allclose(z1, z2, rtol=0, atol=1e-13)
    assert np.allclose(d1, d2, rtol=0, atol=1e-13)


@pytest.mark.parametrize("gz,stretch", [(64, 2.0), (192, 2.0), (48, 4.0)])
def test_tanh_mesh(gz, stretch):
    d1, z1 = mesh.tanh_mesh(gz, 5.0, stretch)
    d2, z2 = of.tanh_mesh(gz, 5.0, stretch)
    assert np.array_equal(z1, z2) and np.allclose(d1, d2, rtol=1e-15, atol=0)


@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_contour_steps(scheme):
    a, b = mesh.contour_steps(150, scheme), of.contour_steps(150, scheme)
    assert a[0] == 0.0 and abs(a.sum() - 1.0) < 1e-14
    assert np.allclose(a, b, rtol=1e-12, atol=0)


@pytest.mark.parametrize("walls", [(True, True), (True, False), (False, True)])
def test_wall_potential(walls):
    dz, zr = of.tanh_mesh(80, 3.0)
    u = mesh.wall_potential(zr, 3.0, 0.5, (0.7, -0.2), walls)
    shape = oi.wall_potential_shape(zr, 3.0, 0.5, walls)
    assert np.allclose(u, np.stack([0.7 * shape, -0.2 * shape]), rtol=0, atol=1e-15)
