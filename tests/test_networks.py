"""Synthetic flow maps: balance, CDF and neighbour tables (03_cma.md)."""
import numpy as np
import pytest

from bmc import networks


@pytest.mark.parametrize("n", [4, 8])
def test_lattice_balanced_and_cdf(n):
    net = networks.lattice_vortex(n, seed=3)
    assert net.n_c == n ** 3
    assert np.abs(net.divergence()).max() < 1e-15
    assert (np.diff(net.cdf, axis=1) >= 0).all()
    assert np.allclose(net.cdf[net.out_flow > 0, -1], 1.0, atol=1e-12)
    assert (net.neighbors < net.n_c).all()
    T = net.transition_dense()
    assert np.allclose(T.sum(axis=1), 0.0, atol=1e-15)  # rows conserve mass
    # destination probabilities equal F(i,j) / sum_k F(i,k)
    i = int(np.argmax(net.out_flow))
    mask = net.src == i
    probs = np.diff(np.concatenate([[0.0], net.cdf[i, : mask.sum()]]))
    assert np.allclose(probs, net.flow[mask] / net.flow[mask].sum())


def test_lattice_peak_velocity():
    net = networks.lattice_vortex(8, side=1.0, peak_velocity=0.5, noise=0.0)
    h = 1.0 / 8
    assert abs(net.flow.max() / (h * h) - 0.5) < 1e-12


def test_ring_balanced_and_courant():
    net = networks.ring_network(10, 2, seed=42, max_courant=0.5, dt=0.1)
    assert np.abs(net.divergence()).max() < 1e-15
    assert net.max_courant(0.1) <= 0.5 + 1e-12
    assert net.K >= 3


def test_single_compartment():
    net = networks.single_compartment()
    assert net.n_c == 1 and net.K == 1 and net.out_flow[0] == 0.0
