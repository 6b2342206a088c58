"""Network reader/writer and the seeded generator (no GPU)."""
import numpy as np
import pytest

from conftest import network_2_7


def test_round_trip_of_the_reference_network(golden_2_7):
    from mumfim_gb300 import network_io as io
    net = network_2_7(golden_2_7)
    coords, conn = io.parse_network(io.format_network(net))
    np.testing.assert_array_equal(coords, net.coords)
    np.testing.assert_array_equal(conn, net.connectivity)
    reactions, fr = io.parse_params(io.format_params(net), net.n_fibers)
    assert reactions[0] == net.reactions[0]
    assert fr.tolist() == [0] * net.n_fibers


def test_params_with_nonlinear_reaction_and_periodic_lines():
    from mumfim_gb300 import network_io as io
    coords, conn = io.parse_network("3 2 1\n0 0 0\n1 0 0\n0 1 0\n0 1\n1 2\n1 3\n")
    assert coords.shape == (3, 3) and conn.tolist() == [[0, 1], [1, 2]]
    reactions, fr = io.parse_params("2 2\n0 5e-05 1e8 1000\n1 1e-3 2.0 4.0 1.05 1.0\n1\n0\n", 2)
    assert reactions[1].law == io.NONLINEAR and reactions[1].B == 4.0
    assert reactions[1].length_ratio_trns == 1.05 and reactions[1].density == 1.0
    assert fr.tolist() == [1, 0]


@pytest.mark.parametrize("text,n", [("3 1 0\n0 0 0\n1 0 0\n0 1 0\n0 3\n", None),
                                    ("2 1 0\n0 0 0\n", None)])
def test_malformed_networks_raise(text, n):
    from mumfim_gb300 import network_io as io
    with pytest.raises(io.NetworkFormatError):
        io.parse_network(text)


def test_params_fiber_count_must_match():
    from mumfim_gb300 import network_io as io
    with pytest.raises(io.NetworkFormatError):
        io.parse_params("1 3\n0 1 1 1\n0\n0\n0\n", 2)


def test_generator_is_deterministic_and_exact_knn(lib_path):
    from mumfim_gb300 import synthetic as S
    c1, e1 = S.knn_network(400, 4, 99)
    c2, e2 = S.knn_network(400, 4, 99)
    np.testing.assert_array_equal(c1, c2)
    np.testing.assert_array_equal(e1, e2)
    d = ((c1[:, None, :] - c1[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d, np.inf)
    nn = np.argsort(d, axis=1, kind="stable")[:, :4]
    ref = {(min(i, j), max(i, j)) for i in range(400) for j in nn[i]}
    assert ref == set(map(tuple, e1.tolist()))
    # face snapping: a coordinate is either exactly +-0.5 or at least 0.02 inside
    a = np.abs(c1)
    assert np.all((a == 0.5) | (a < 0.5 - 0.02))
    assert np.min(d) >= 1e-12


def test_portable_exp_log_accuracy(lib_path):
    from mumfim_gb300 import synthetic as S
    for x in (-20.0, -3.3, -1e-9, 0.0, 0.7, 5.5, 40.0):
        assert abs(S.pexp(x) - np.exp(x)) <= 4e-16 * np.exp(x)
    for x in (1e-300, 1e-3, 0.5, 1.0, 2.0, 12345.678):
        assert abs(S.plog(x) - np.log(x)) <= 4e-16 * max(1.0, abs(np.log(x)))


def test_config_shapes(lib_path):
    from mumfim_gb300 import synthetic as S
    w = S.config0()
    assert w.n_rve == 1 and w.networks[0].n_nodes == 1000 and 2300 < w.total_fibers < 2800
    assert w.strategies[0].mode == 1 and w.steps == 10_000
    w = S.config2(n_rve=64)
    n = [x.n_nodes for x in w.networks]
    assert 500 <= min(n) and max(n) <= 20_000
    assert np.all(np.abs(w.F - np.eye(3)) <= 0.08)
    w = S.config3(n_rve=8, n_min=300, n_max=400)
    r = w.networks[0].reactions[0]
    assert r.law == 1 and 1.0 <= r.B <= 10.0 and 1.02 <= r.length_ratio_trns <= 1.15
