"""The oracle against the reference's unit-test known answers.

Each test restates one assertion of diffmpm's own unit tests (file:line cited)
on the NumPy oracle.  The tolerance is ``jnp.allclose``'s default (rtol 1e-5,
atol 1e-8), as in the reference.
"""
import numpy as np
import pytest

from oracle.mpm_oracle import (Constraint, LinearElastic, NodalForce, Particles,
                               Quadrilateral4Node, SimpleMaterial, Unit)


def allclose(a, b):
    return np.allclose(np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64))


@pytest.fixture
def elements():
    # tests/test_element.py:17-19
    return Quadrilateral4Node((1, 1), 1, (1.0, 1.0), [])


@pytest.fixture
def particles():
    # tests/test_element.py:21-25
    loc = np.array([[0.5, 0.5], [0.5, 0.5]]).reshape(2, 1, 2)
    return Particles(loc, SimpleMaterial({"E": 1, "density": 1}), np.array([0, 0]))


# --- tests/test_element.py ---------------------------------------------------
@pytest.mark.parametrize("coords, expected", [
    (np.array([[0, 0]]).reshape(-1, 1, 2), np.array([0.25, 0.25, 0.25, 0.25]).reshape(1, 4, 1, 1)),
    (np.array([[-1, -1]]).reshape(-1, 1, 2), np.array([1, 0, 0, 0]).reshape(1, 4, 1, 1)),
    (np.array([[1, 1]]).reshape(-1, 1, 2), np.array([0, 0, 1, 0]).reshape(1, 4, 1, 1)),
])
def test_shapefn(elements, coords, expected):
    # tests/test_element.py:27-46
    assert allclose(elements.shapefn(coords.astype(np.float32)), expected)


@pytest.mark.parametrize("coords, expected", [
    (np.array([[0, 0]]).reshape(-1, 1, 2),
     np.array([[-0.25, -0.25], [0.25, -0.25], [0.25, 0.25], [-0.25, 0.25]]).reshape(-1, 4, 2)),
    (np.array([[-1, -1]]).reshape(-1, 1, 2),
     np.array([[-0.5, -0.5], [0.5, 0.0], [0.0, 0.0], [0.0, 0.5]]).reshape(-1, 4, 2)),
    (np.array([[1, 1]]).reshape(-1, 1, 2),
     np.array([[0.0, 0.0], [0.0, -0.5], [0.5, 0.5], [-0.5, 0.0]]).reshape(-1, 4, 2)),
])
def test_shapefn_natural_grad(elements, coords, expected):
    # tests/test_element.py:48-73
    assert allclose(elements._shapefn_natural_grad(coords.astype(np.float32)), expected)


@pytest.mark.parametrize("coords", [
    np.array([[0.5, 0.5]]).reshape(-1, 1, 2),
    np.array([[-0.5, -0.5]]).reshape(-1, 1, 2),
])
def test_shapefn_grad(elements, coords):
    # tests/test_element.py:75-88: on a unit element dN/dx = 2 dN/dxi
    coords = coords.astype(np.float32)
    nodal = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]]).reshape(-1, 4, 2)
    expected = elements._shapefn_natural_grad(coords) * 2
    assert allclose(elements.shapefn_grad(coords, nodal), expected)
    # the axis-aligned specialisation the step uses gives the same answer
    assert allclose(elements.dn_dx(coords, np.array([0])), expected)


def test_element_node_ids(elements):
    # tests/test_element.py:90-94
    assert np.all(elements.id_to_node_ids(0).reshape(-1) == np.array([0, 1, 3, 2]))


def test_element_node_loc(elements):
    # tests/test_element.py:96-99
    true_loc = np.array([[0.0, 0.0], [1, 0], [1, 1], [0, 1]]).reshape(4, 1, 2)
    assert np.all(elements.id_to_node_loc(0) == true_loc)


def test_element_node_vel(elements):
    # tests/test_element.py:101-105
    elements.nodes.velocity += np.array([1, 1], dtype=np.float32)
    assert np.all(elements.id_to_node_vel(0) == np.ones((4, 1, 2)))


def test_compute_nodal_mass(elements, particles):
    # tests/test_element.py:107-111
    particles.mass += 1
    elements.compute_nodal_mass(particles)
    assert np.all(elements.nodes.mass == np.ones((4, 1, 1)))


def test_compute_nodal_momentum(elements, particles):
    # tests/test_element.py:113-117
    particles.velocity += 1
    elements.compute_nodal_momentum(particles)
    assert np.all(elements.nodes.momentum == np.ones((4, 1, 1)) * 0.5)


def test_compute_external_force(elements, particles):
    # tests/test_element.py:119-123
    particles.f_ext += 1
    elements.compute_external_force(particles)
    assert np.all(elements.nodes.f_ext == np.ones((4, 1, 1)) * 0.5)


@pytest.mark.parametrize("gravity, expected", [
    (0, np.zeros((4, 1, 2))),
    (np.array([10, 0]), np.array([[10, 0], [10, 0], [10, 0], [10, 0]]).reshape(4, 1, 2)),
])
def test_compute_body_force(elements, particles, gravity, expected):
    # tests/test_element.py:125-138
    particles.mass += 1
    elements.compute_body_force(particles, gravity)
    assert np.all(elements.nodes.f_ext == expected)


def test_apply_concentrated_nodal_force(particles):
    # tests/test_element.py:140-160
    cnf_1 = NodalForce(node_ids=np.array([0, 2]), function=Unit(-1), dir=0, force=1)
    cnf_2 = NodalForce(node_ids=np.array([2]), function=Unit(-1), dir=1, force=1)
    elements = Quadrilateral4Node((1, 1), 1, 1, [], concentrated_nodal_forces=[cnf_1, cnf_2])
    elements.apply_concentrated_nodal_forces(particles, 1)
    assert np.all(elements.nodes.f_ext == np.array([[1, 0], [0, 0], [1, 1], [0, 0]]).reshape(4, 1, 2))


def test_apply_boundary_constraints():
    # tests/test_element.py:162-170
    cons = [(np.array([0]), Constraint(0, 0))]
    elements = Quadrilateral4Node((1, 1), 1, (1.0, 1.0), cons)
    elements.nodes.velocity += 1
    elements.apply_boundary_constraints()
    assert np.all(elements.nodes.velocity == np.array([[0, 1], [1, 1], [1, 1], [1, 1]]).reshape(4, 1, 2))


def test_update_nodal_acceleration_velocity(elements, particles):
    # tests/test_element.py:172-187
    elements.nodes.f_ext += np.array([1, 0], dtype=np.float32)
    elements.nodes.mass[:] = 2
    elements.update_nodal_acceleration_velocity(particles, 0.1)
    assert allclose(elements.nodes.acceleration, np.array([[0.5, 0.0]] * 4).reshape(4, 1, 2))
    assert allclose(elements.nodes.velocity, np.array([[0.05, 0.0]] * 4).reshape(4, 1, 2))
    assert allclose(elements.nodes.momentum, np.array([[0.1, 0.0]] * 4).reshape(4, 1, 2))


def test_set_particle_element_ids(elements, particles):
    # tests/test_element.py:189-192
    particles.element_ids = np.array([-1, -1])
    elements.set_particle_element_ids(particles)
    assert np.all(particles.element_ids == np.array([0, 0]))


def test_compute_internal_force(elements, particles):
    # tests/test_element.py:194-201
    particles.compute_volume(elements, 1)
    particles.stress += 1
    elements.compute_internal_force(particles)
    assert allclose(elements.nodes.f_int, np.array([[1, 1], [0, 0], [0, 0], [-1, -1]]).reshape(4, 1, 2))


def test_compute_volume(elements):
    # tests/test_element.py:203-205
    elements.compute_volume()
    assert allclose(elements.volume, np.array([1]).reshape(1, 1, 1))


def test_apply_particle_traction_forces(elements, particles):
    # tests/test_element.py:207-212
    particles.traction += np.array([1, 0], dtype=np.float32)
    elements.apply_particle_traction_forces(particles)
    assert allclose(elements.nodes.f_ext, np.array([[0.5, 0]] * 4).reshape(4, 1, 2))


# --- tests/test_particle.py --------------------------------------------------
@pytest.mark.parametrize("velocity_update, expected", [
    (False, np.array([[0.1, 0.1], [0.1, 0.1]]).reshape(2, 1, 2)),
    (True, np.array([[1, 1], [1, 1]]).reshape(2, 1, 2)),
])
def test_update_velocity(elements, particles, velocity_update, expected):
    # tests/test_particle.py:33-45
    particles.update_natural_coords(elements)
    elements.nodes.acceleration += 1
    elements.nodes.velocity += 1
    particles.update_position_velocity(elements, 0.1, velocity_update)
    assert allclose(particles.velocity, expected)


def test_compute_strain(elements, particles):
    # tests/test_particle.py:47-59
    elements.nodes.velocity = np.array([[0, 1], [0, 2], [0, 3], [0, 4]], dtype=np.float32).reshape(4, 1, 2)
    particles.update_natural_coords(elements)
    particles.compute_strain(elements, 0.1)
    assert allclose(particles.strain,
                    np.array([[0, 0.2, 0, 0.1, 0, 0], [0, 0.2, 0, 0.1, 0, 0]]).reshape(2, 6, 1))
    assert allclose(particles.volumetric_strain_centroid, np.array([0.2]))


def test_particle_compute_volume(elements, particles):
    # tests/test_particle.py:61-63
    particles.compute_volume(elements, elements.total_elements)
    assert allclose(particles.volume, np.array([0.5, 0.5]).reshape(2, 1, 1))


def test_assign_traction(elements, particles):
    # tests/test_particle.py:65-70
    particles.compute_volume(elements, elements.total_elements)
    particles.assign_traction(np.array([0]), 1, 10)
    assert allclose(particles.traction, np.array([[0, 7.071068], [0, 0]]).reshape(2, 1, 2))


def test_zero_traction(particles):
    # tests/test_particle.py:72-75
    particles.traction += 1
    particles.zero_traction()
    assert np.all(particles.traction == 0)


# --- tests/test_material.py --------------------------------------------------
@pytest.mark.parametrize("material, dstrain, target", [
    (SimpleMaterial({"E": 10, "density": 1}), np.ones((1, 6, 1)), np.ones((1, 6, 1)) * 10),
    (LinearElastic({"density": 1, "youngs_modulus": 10, "poisson_ratio": 1}), np.ones((1, 6, 1)),
     np.array([-10, -10, -10, 2.5, 2.5, 2.5]).reshape(1, 6, 1)),
    (LinearElastic({"density": 1000, "youngs_modulus": 1e7, "poisson_ratio": 0.3}),
     np.array([0.001, 0.0005, 0, 0, 0, 0]).reshape(1, 6, 1),
     np.array([1.63461538461538e4, 12500, 0.86538461538462e4, 0, 0, 0]).reshape(1, 6, 1)),
    (LinearElastic({"density": 1000, "youngs_modulus": 1e7, "poisson_ratio": 0.3}),
     np.array([0.001, 0.0005, 0, 0.00001, 0, 0]).reshape(1, 6, 1),
     np.array([1.63461538461538e4, 12500, 0.86538461538462e4, 3.84615384615385e01, 0, 0]).reshape(1, 6, 1)),
])
def test_compute_stress(material, dstrain, target):
    # tests/test_material.py:6-37
    assert allclose(material.compute_stress(dstrain.astype(np.float32)), target)


def test_linear_elastic_missing_prop():
    # material.py:45-51 raises KeyError for a missing property
    with pytest.raises(KeyError):
        LinearElastic({"density": 1, "youngs_modulus": 10})


def test_shapefn_rejects_bad_rank(elements):
    # element.py:743-747
    with pytest.raises(ValueError):
        elements.shapefn(np.zeros((2, 2), dtype=np.float32))
