"""The uneven-block workload: a random 3-D tight-binding graph sliced by BFS layers
(slice_1contact, src/graph_partition.f90:282-316,426-450).  Blocks checked against a
dense H(k) built from all atom pairs at once."""
import numpy as np

from quantum_transport_gb300.devices import bfs_layers, config_uneven


def dense_h(natoms, box, cutoff, seed, k):
    """H(k) over all pairs with the minimum image along y, atoms in input order."""
    rng = np.random.default_rng(seed)
    L = np.asarray(box)
    pos = rng.uniform(0.0, 1.0, (natoms, 3)) * L
    onsite = rng.normal(0.0, 0.2, natoms)
    d = pos[None, :, :] - pos[:, None, :]
    w = -np.round(d[..., 1] / L[1])
    d[..., 1] += w * L[1]
    r = np.sqrt((d * d).sum(-1))
    bond = (r < cutoff) & ~np.eye(natoms, dtype=bool)
    H = np.where(bond, -2.7 * np.exp(-3.0 * (r / 1.42 - 1.0)) * np.exp(1j * k * w), 0.0)
    return H + np.diag(onsite)


def test_blocks_match_dense_hamiltonian():
    natoms, box, cutoff, seed = 800, (12.0, 6.0, 6.0), 2.6, 11
    d = config_uneven(seed=seed, natoms=natoms, box=box, nE=4, nk=4)
    assert sum(d.sizes) == natoms and d.nx >= 3
    for ik, k in enumerate(d.kpts):
        H = dense_h(natoms, box, cutoff, seed, k)[np.ix_(d.order, d.order)]
        off = np.concatenate([[0], np.cumsum(d.sizes)])
        for l in range(d.nx):
            s = slice(off[l], off[l + 1])
            np.testing.assert_allclose(d.Hii[l][ik], H[s, s], atol=1e-13)
            if l:
                p = slice(off[l - 1], off[l])
                np.testing.assert_allclose(d.H1i[l][ik], H[s, p], atol=1e-13)
            for m in range(l + 2, d.nx):  # nothing beyond the neighbouring slab
                assert not H[s, off[m]:off[m + 1]].any()


def test_benchmark_partition():
    d = config_uneven(nE=2)
    assert sum(d.sizes) == 4000 and 20 <= d.nx <= 30
    assert min(d.sizes) > 128 and max(d.sizes) <= 384  # every block needs the tiled split path
    assert d.H1i[0].shape == (8, d.sizes[0], d.sizes[0])


def test_bfs_layers_distance():
    # a path 0-1-2-3 plus a branch 1-4: distances from {0}
    D = bfs_layers(5, [(0, 1), (1, 2), (2, 3), (1, 4)], np.array([0]))
    assert list(D) == [0, 1, 2, 3, 2]
