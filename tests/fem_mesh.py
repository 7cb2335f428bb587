"""A structured HEX20 dof map for the FEM point-value tests: the nodes of a
uniform box mesh on the (2nx+1) x (2ny+1) x (2nz+1) lattice, libMesh Hex20
node order per element, u/v/w dofs shuffled by a seeded permutation (the
driver's DofMap numbering is arbitrary)."""
import numpy as np

HEX20 = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                  [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1],
                  [0, -1, -1], [1, 0, -1], [0, 1, -1], [-1, 0, -1],
                  [-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0],
                  [0, -1, 1], [1, 0, 1], [0, 1, 1], [-1, 0, 1]])


def hex20_mesh(ne, lo, hi, seed=0):
    """(elem_dofs [n_elem][3][20], n_dofs, lattice xyz of every dof)"""
    ne = np.asarray(ne)
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    nl = 2 * ne + 1
    ex, ey, ez = np.meshgrid(np.arange(ne[0]), np.arange(ne[1]), np.arange(ne[2]), indexing="ij")
    # elements x fastest (build_cube order)
    E = np.stack([ex.transpose(2, 1, 0).ravel(), ey.transpose(2, 1, 0).ravel(),
                  ez.transpose(2, 1, 0).ravel()], axis=1)
    lat = 2 * E[:, None, :] + 1 + HEX20[None, :, :]                      # [ne][20][3]
    node = lat[..., 0] + nl[0] * (lat[..., 1] + nl[1] * lat[..., 2])     # lattice node id
    n_nodes = int(np.prod(nl))
    perm = np.random.default_rng(seed).permutation(3 * n_nodes)
    dofs = np.stack([perm[3 * node + v] for v in range(3)], axis=1)      # [ne][3][20]
    # position of every dof (for nodal values of a field)
    ids = np.arange(n_nodes)
    lx, ly, lz = ids % nl[0], (ids // nl[0]) % nl[1], ids // (nl[0] * nl[1])
    h = (hi - lo) / ne
    pos = lo + np.stack([lx, ly, lz], axis=1) * (h / 2)
    dof_pos = np.zeros((3 * n_nodes, 3))
    dof_var = np.zeros(3 * n_nodes, dtype=int)
    for v in range(3):
        dof_pos[perm[3 * ids + v]] = pos
        dof_var[perm[3 * ids + v]] = v
    return dofs, 3 * n_nodes, dof_pos, dof_var


def quadratic(x, v):
    """a complete quadratic in (x, y, z), different for each variable v"""
    c = np.array([[0.3, -1.1, 0.7], [1.2, 0.4, -0.5], [-0.8, 0.9, 0.2]])[v]
    X, Y, Z = x[..., 0], x[..., 1], x[..., 2]
    return (0.5 + c[0] * X + c[1] * Y + c[2] * Z + 0.01 * c[0] * X * X - 0.02 * Y * Y
            + 0.015 * Z * Z + 0.03 * X * Y - 0.01 * c[1] * Y * Z + 0.02 * Z * X)
