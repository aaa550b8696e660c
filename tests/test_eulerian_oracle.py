"""The oracle's restatement of the grid metrics and Contra2Cart (oracle/picurv_oracle.c)
against an independent numpy restatement (tests/pyref_metrics.py), bit for bit, plus
known answers: a uniform grid's metrics are its face areas and volume, a uniform flow
comes back exactly, a left-handed grid is flipped, and the reference's three errors.
CPU only."""
import numpy as np
import pytest

from fdf_gb300 import workloads as W
from oracle import oracle as O
from tests import pyref_metrics as R


def _grids():
    return {
        "sinusoidal": W.sinusoidal_grid(8, 6, 10),
        "bent_pipe": W.bent_pipe_grid(6, 6, 12),
        "curved_pipe": W.curved_pipe_grid(6, 6, 10),
        "thin": W.sinusoidal_grid(1, 3, 2),
    }


@pytest.mark.parametrize("name", list(_grids()))
def test_metrics_match_numpy_restatement(name):
    coor = _grids()[name]
    got = O.grid_metrics(O.Grid(coor))
    ref = R.metrics(coor)
    for a, b, what in zip(got[:4], ref[:4], ("csi", "eta", "zet", "aj")):
        assert np.array_equal(a, b), f"{name}: {what} differs"
    assert got[4] == ref[4] is False


@pytest.mark.parametrize("name", list(_grids()))
def test_contra2cart_matches_numpy_restatement(name):
    coor = _grids()[name]
    g = O.Grid(coor)
    csi, eta, zet, _, _ = O.grid_metrics(g)
    rng = np.random.default_rng(7)
    ucont = rng.uniform(-1.0, 1.0, size=coor.shape)
    ucat0 = rng.uniform(-1.0, 1.0, size=coor.shape)
    got = O.contra2cart(g, ucont, csi, eta, zet, ucat0)
    ref = R.contra2cart(ucont, csi, eta, zet, ucat0)
    assert np.array_equal(got, ref)
    # only the interior cells change
    mask = np.zeros(coor.shape[:3], dtype=bool)
    mask[1:-1, 1:-1, 1:-1] = True
    assert np.array_equal(got[~mask], ucat0[~mask])


def test_uniform_grid_known_answers():
    IM, JM, KM = 4, 8, 2
    coor = W.uniform_grid(IM, JM, KM)     # spacings 1/4, 1/8, 1/2: every product is exact
    hx, hy, hz = 1.0 / IM, 1.0 / JM, 1.0 / KM
    csi, eta, zet, aj, flipped = O.grid_metrics(O.Grid(coor))
    assert not flipped
    assert np.all(csi == np.array([hy * hz, 0.0, 0.0]))
    assert np.all(eta == np.array([0.0, hx * hz, 0.0]))
    assert np.all(zet == np.array([0.0, 0.0, hx * hy]))
    assert np.all(aj == 1.0 / (hx * hy * hz))
    u = np.array([0.75, -1.5, 2.0])
    ucont = R.ucont_of_uniform_flow(u, csi, eta, zet)
    ucat = O.contra2cart(O.Grid(coor), ucont, csi, eta, zet)
    assert np.array_equal(ucat[1:KM, 1:JM, 1:IM], np.broadcast_to(u, (KM - 1, JM - 1, IM - 1, 3)))
    assert not ucat[0].any() and not ucat[:, :, IM].any()


def test_uniform_flow_on_curvilinear_grid_is_recovered():
    coor = W.bent_pipe_grid(8, 8, 16)
    g = O.Grid(coor)
    csi, eta, zet, _, _ = O.grid_metrics(g)
    u = np.array([0.3, -0.2, 1.1])
    ucat = O.contra2cart(g, R.ucont_of_uniform_flow(u, csi, eta, zet), csi, eta, zet)
    err = np.abs(ucat[1:-1, 1:-1, 1:-1] - u).max()
    assert err < 1e-13 * np.abs(u).max(), err


def test_left_handed_grid_is_flipped():
    coor = W.sinusoidal_grid(6, 5, 8)
    lh = np.ascontiguousarray(coor[::-1])          # k reversed: every Jacobian negative
    csi, eta, zet, aj, flipped = O.grid_metrics(O.Grid(lh))
    assert flipped and np.all(aj > 0)
    raw = R.face_metrics(lh)
    assert np.array_equal(csi, -raw[0]) and np.array_equal(eta, -raw[1]) and np.array_equal(zet, -raw[2])
    ref = R.metrics(lh)
    assert ref[4] is True and np.array_equal(ref[3], aj)
    # Contra2Cart with the flipped metrics still returns the flow that made the fluxes
    u = np.array([0.5, 0.25, -1.0])
    ucat = O.contra2cart(O.Grid(lh), R.ucont_of_uniform_flow(u, csi, eta, zet), csi, eta, zet)
    assert np.abs(ucat[1:-1, 1:-1, 1:-1] - u).max() < 1e-13


def folded_grid():
    """A grid whose z coordinate runs back after k = 2: Jacobians of both signs, none near zero."""
    coor = W.uniform_grid(3, 3, 4).copy()
    z = np.array([0.0, 0.25, 0.5, 0.25, 0.0])
    coor[..., 2] = z[:, None, None]
    return coor


def collapsed_grid():
    """Node plane k = 1 on top of k = 0: zero Jacobian at the nodes of k = 1."""
    coor = W.uniform_grid(3, 3, 4).copy()
    coor[1] = coor[0]
    return coor


def test_mixed_orientation_is_an_error():
    with pytest.raises(O.OracleError) as e:
        O.grid_metrics(O.Grid(folded_grid()))
    assert e.value.code == O.ERR_USER
    with pytest.raises(R.MetricError) as e2:
        R.metrics(folded_grid())
    assert e2.value.code == 83


def test_zero_jacobian_is_an_error():
    with pytest.raises(O.OracleError) as e:
        O.grid_metrics(O.Grid(collapsed_grid()))
    assert e.value.code == O.ERR_FLOP_COUNT
    with pytest.raises(R.MetricError):
        R.jacobian_inverse(collapsed_grid())


def test_near_zero_determinant_is_an_error():
    coor = W.uniform_grid(3, 3, 3) * 5e-4   # |J| = 1.25e-10 passes, |det| ~ 1.6e-20 does not
    g = O.Grid(coor)
    csi, eta, zet, _, _ = O.grid_metrics(g)
    with pytest.raises(O.OracleError) as e:
        O.contra2cart(g, np.zeros(coor.shape), csi, eta, zet)
    assert e.value.code == O.ERR_FLOP_COUNT
