"""Local MLIAP energy in float64 (oracle, test infrastructure).

Restates ``local_mliap_energy_full`` (src/kups/potential/mliap/local.py:310-356): node
embeddings init(Z), messages edge(h_i, h_j, d_ij) over the full directed neighbour list
(``oracle.neighborlist``, reference-exact), sums onto the first atom, readout per atom,
sums per system.  ``simple_model`` is the model of the reference's tests
(test/potential/test_local_mliap.py:51-67): embedding 0.1 for every species and feature,
message h_j / (|d| + 1), readout 0.1 * sum(h + m).
"""

from __future__ import annotations

import numpy as np

from .neighborlist import neighbor_list
from .unitcell import lattice_from_tril


def simple_model(embed_dim: int = 4, n_species: int = 3, xp=np):
    embedding = xp.ones((n_species, embed_dim)) * 0.1
    readout_w = xp.ones((embed_dim, 1)) * 0.1

    def init_function(z):
        return embedding[z]

    def edge_function(h1, h2, d):
        dist = (d * d).sum(-1, keepdims=True) ** 0.5
        return h2 / (dist + 1.0)

    def readout_function(h, m):
        return ((h + m) @ readout_w)[..., 0]

    return init_function, edge_function, readout_function


def local_mliap_energy(model, pos, z, system, tril, cutoffs):
    """(energy [S], node embeddings [N, F], message sums [N, F'])."""
    init_fn, edge_fn, readout_fn = model
    pos = np.asarray(pos, np.float64)
    system = np.asarray(system)
    tril = np.asarray(tril, np.float64)
    e, s = neighbor_list(pos, system, tril, cutoffs)
    L = lattice_from_tril(tril)[system[e[:, 0]]]
    d = pos[e[:, 1]] - pos[e[:, 0]] + np.einsum("ek,ekl->el", s.astype(np.float64), L)
    h = init_fn(np.asarray(z))
    m = edge_fn(h[e[:, 0]], h[e[:, 1]], d)
    msg = np.zeros((len(pos),) + m.shape[1:])
    np.add.at(msg, e[:, 0], m)
    ea = readout_fn(h, msg)
    energy = np.zeros(tril.shape[0])
    np.add.at(energy, system, ea)
    return energy, h, msg
