"""The coordinate front end (hera_gpu_gb300/sky.py): (LST, latitude) ->
eq2top rotations and (RA, Dec) -> crd_eq, the inputs hera_gpu's vis_gpu
takes ready-made (hera_gpu/vis.py:144).  CPU only.

Checked against the spherical-astronomy relations for hour angle
H = LST - RA and latitude phi, written out here independently of the
module's matrix:
    east  = -cos(Dec) sin(H)
    north =  cos(phi) sin(Dec) - sin(phi) cos(Dec) cos(H)
    up    =  sin(phi) sin(Dec) + cos(phi) cos(Dec) cos(H)
and against directions whose position is known without them.
"""
import numpy as np
import pytest

from hera_gpu_gb300 import sky


def topocentric(lst, lat, ra, dec):
    h = lst - ra
    return np.stack([-np.cos(dec) * np.sin(h),
                     np.cos(lat) * np.sin(dec) - np.sin(lat) * np.cos(dec) * np.cos(h),
                     np.sin(lat) * np.sin(dec) + np.cos(lat) * np.cos(dec) * np.cos(h)])


@pytest.mark.parametrize("seed", range(4))
def test_eq2top_is_a_rotation(seed):
    rng = np.random.default_rng(seed)
    r = sky.eq2top(rng.uniform(0, 2 * np.pi), rng.uniform(-np.pi / 2, np.pi / 2))
    np.testing.assert_allclose(r @ r.T, np.identity(3), atol=1e-15)
    assert np.linalg.det(r) == pytest.approx(1.0, abs=1e-14)


def test_eq2top_matches_the_hour_angle_relations():
    rng = np.random.default_rng(10)
    ra = rng.uniform(0, 2 * np.pi, 500)
    dec = np.arcsin(rng.uniform(-1, 1, 500))
    crd = sky.radec_to_crd_eq(ra, dec)
    for lst, lat in zip(rng.uniform(0, 2 * np.pi, 6), rng.uniform(-np.pi / 2, np.pi / 2, 6)):
        np.testing.assert_allclose(sky.eq2top(lst, lat) @ crd, topocentric(lst, lat, ra, dec),
                                   atol=1e-14)


@pytest.mark.parametrize("lat_deg", [sky.HERA_LATITUDE_DEG, 0.0, 52.0, -89.0])
def test_known_directions(lat_deg):
    lat, lst = np.radians(lat_deg), 1.234
    r = sky.eq2top(lst, lat)
    # a source on the meridian at Dec = latitude is at the zenith
    np.testing.assert_allclose(r @ sky.radec_to_crd_eq(lst, lat), [0, 0, 1], atol=1e-15)
    # the north celestial pole: due north, altitude = latitude
    np.testing.assert_allclose(r @ [0, 0, 1], [0, np.cos(lat), np.sin(lat)], atol=1e-15)
    # on the meridian 30 degrees south of the zenith
    np.testing.assert_allclose(r @ sky.radec_to_crd_eq(lst, lat - np.radians(30)),
                               [0, -0.5, np.cos(np.radians(30))], atol=1e-15)
    # six sidereal hours before transit, on the equator: due east on the horizon
    np.testing.assert_allclose(r @ sky.radec_to_crd_eq(lst + np.pi / 2, 0.0), [1, 0, 0],
                               atol=1e-15)


def test_sky_turns_once_per_sidereal_day():
    lat = np.radians(sky.HERA_LATITUDE_DEG)
    np.testing.assert_allclose(sky.eq2top(0.3 + 2 * np.pi, lat), sky.eq2top(0.3, lat),
                               atol=1e-15)
    # a source rises in the east: its east component falls as the LST grows
    # through its rising, and it transits when LST = RA
    crd = sky.radec_to_crd_eq(2.0, np.radians(-30.0))
    lsts = sky.lst_grid(7, hours=12.0, start_rad=2.0 - np.pi / 2)
    top = np.einsum("tij,j->ti", sky.eq2tops(lsts, lat), crd)
    assert np.all(np.diff(top[:, 0]) < 0)
    assert np.argmax(top[:, 2]) == 3 and lsts[3] == pytest.approx(2.0)


def test_radec_to_crd_eq_axes():
    crd = sky.radec_to_crd_eq(np.array([0.0, np.pi / 2, 1.0]), np.array([0.0, 0.0, np.pi / 2]))
    np.testing.assert_allclose(crd, [[1, 0, 0], [0, 1, 0], [0, 0, 1]], atol=1e-15)
    rng = np.random.default_rng(3)
    crd = sky.radec_to_crd_eq(rng.uniform(0, 7, 100), rng.uniform(-2, 2, 100))
    np.testing.assert_allclose(np.linalg.norm(crd, axis=0), 1, atol=1e-15)


def test_lst_grid_and_stack():
    g = sky.lst_grid(5, hours=2.0, start_rad=0.5)
    np.testing.assert_allclose(g, 0.5 + np.linspace(0, 2 / 24 * 2 * np.pi, 5))
    np.testing.assert_array_equal(sky.lst_grid(1, start_rad=0.7), [0.7])
    e = sky.eq2tops(g, 0.1)
    assert e.shape == (5, 3, 3)
    np.testing.assert_array_equal(e[2], sky.eq2top(g[2], 0.1))


# HERA simulators build eq2tops with aipy's coordinate convention,
# eq2top_m(ha, dec) evaluated at ha = -LST and dec = latitude: the passive
# rotation R_x(pi/2 - dec) R_z(pi/2 - ha) (R_z turns the x axis to the east
# of the meridian, R_x tilts the pole to the observer's latitude).  Golden
# values of that convention, computed from the rotation product and rounded
# to 15 digits: (LST rad, latitude deg) -> matrix.
AIPY_CONVENTION_GOLDEN = {
    (0.0, -30.72): [[0.0, 1.0, 0.0], [0.51084303186586, 0.0, 0.859674006117491],
                    [0.859674006117491, 0.0, -0.51084303186586]],
    (1.0, -30.72): [[-0.841470984807896, 0.54030230586814, 0.0],
                    [0.276009668053796, 0.429859589106417, 0.859674006117491],
                    [0.464483847800182, 0.723390732541435, -0.51084303186586]],
    (4.2, 52.0): [[0.871575772413588, -0.4902608213407, 0.0],
                  [0.386330799288535, 0.686811081244992, 0.615661475325658],
                  [-0.301834700560984, -0.53659562590225, 0.788010753606722]],
    (2.5, 0.0): [[-0.598472144103956, -0.801143615546934, 0.0], [0.0, 0.0, 1.0],
                 [-0.801143615546934, 0.598472144103956, 0.0]],
}


def _rot_x(b):
    c, s = np.cos(b), np.sin(b)
    return np.array([[1.0, 0.0, 0.0], [0.0, c, s], [0.0, -s, c]])


def _rot_z(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[c, s, 0.0], [-s, c, 0.0], [0.0, 0.0, 1.0]])


@pytest.mark.parametrize("key", sorted(AIPY_CONVENTION_GOLDEN))
def test_eq2top_is_the_aipy_convention_of_hera_callers(key):
    lst, lat_deg = key
    got = sky.eq2top(lst, np.radians(lat_deg))
    np.testing.assert_allclose(got, AIPY_CONVENTION_GOLDEN[key], atol=2e-15)
    ha, dec = -lst, np.radians(lat_deg)
    np.testing.assert_allclose(got, _rot_x(np.pi / 2 - dec) @ _rot_z(np.pi / 2 - ha), atol=1e-15)
