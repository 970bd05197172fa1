"""Free/Dirichlet dof numbering of the H1-HDiv spaces (u Q2, p dP1, j RT1, φ dQ1).

Host-side mirror of ``setup_fe_spaces`` / ``fe_space_u|p|j|φ``
(GridapMHD src/fespaces.jl:13-114) with the consecutive multi-field style
(src/fespaces.jl:5): the global free vector is [u; p; j; φ].

Numbering rule (a restatement of Gridap's face-ordered conforming numbering):
dofs are owned by mesh entities, entities are ordered by dimension (vertices,
edges, faces, cells) and lexicographically inside a dimension, and the own
dofs of an entity are consecutive (the 3 velocity components of a Lagrange
node; the 4 normal-flux dofs of an RT face).  Free dofs get ids 0,1,..;
Dirichlet dofs get their own numbering, stored as -(id+1).

The per-cell local layout of 129 dofs is the one the kernels and the oracle
use (u component-major 3x27, p 4, j 36, φ 8); see ``LOCAL_LAYOUT``.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Optional, Sequence

import numpy as np

from .mesh import FACE_AXIS, FACE_SIDE, StructuredMesh

NU, NP, NJ, NPHI = 81, 4, 36, 8
OU, OP, OJ, OPHI = 0, 81, 85, 121
NDOF_CELL = 129
LOCAL_LAYOUT = dict(u=(OU, NU), p=(OP, NP), j=(OJ, NJ), phi=(OPHI, NPHI))

# RT1 local dof b = d*12 + q + 3*(l1 + 2*l2): quadratic index q along axis d,
# linear indices l1, l2 along the two other axes (increasing order).
RT_AXIS = np.repeat(np.arange(3), 12)
RT_Q = np.array([(b % 12) % 3 for b in range(36)])
RT_L = np.array([(b % 12) // 3 for b in range(36)])  # l1 + 2*l2


@dataclass
class DofMap:
    ncells: int
    cell_dofs: np.ndarray         # (ncells, 129) int32, field-local ids, <0 Dirichlet
    nfree: dict                   # field -> number of free dofs
    ndir: dict                    # field -> number of Dirichlet dofs
    dir_values: dict              # field -> float64 array of Dirichlet values
    u_node_coords: np.ndarray     # (nfree_u//3, 3) physical coords of free u nodes
    offsets: dict                 # field -> offset in the global free vector

    @property
    def ndofs(self) -> int:
        return int(sum(self.nfree.values()))

    def global_cell_dofs(self) -> np.ndarray:
        """(ncells,129) int64 global free ids, -1 for Dirichlet slots."""
        g = np.full(self.cell_dofs.shape, -1, dtype=np.int64)
        for f, (o, n) in LOCAL_LAYOUT.items():
            loc = self.cell_dofs[:, o:o + n].astype(np.int64)
            g[:, o:o + n] = np.where(loc >= 0, loc + self.offsets[f], -1)
        return g

    def split(self, x: np.ndarray) -> dict:
        return {f: x[self.offsets[f]:self.offsets[f] + self.nfree[f]] for f in ("u", "p", "j", "phi")}

    def cell_values(self, x: np.ndarray) -> np.ndarray:
        """(ncells,129) local values of the free vector x plus Dirichlet values."""
        out = np.zeros(self.cell_dofs.shape)
        for f, (o, n) in LOCAL_LAYOUT.items():
            loc = self.cell_dofs[:, o:o + n].astype(np.int64)
            xf = x[self.offsets[f]:self.offsets[f] + self.nfree[f]]
            dv = self.dir_values.get(f, np.zeros(0))
            free = loc >= 0
            out[:, o:o + n][free] = xf[loc[free]]
            if (~free).any():
                out[:, o:o + n][~free] = dv[-loc[~free] - 1]
        return out


def _lattice_keys(mesh: StructuredMesh, I, J, K):
    nx, ny, nz = mesh.shape
    dims = [2 * nx, 2 * ny, 2 * nz]
    coords = [np.asarray(I), np.asarray(J), np.asarray(K)]
    for d in range(3):
        if mesh.periodic[d]:
            coords[d] = coords[d] % dims[d]
    NI, NJ_ = 2 * nx + 1, 2 * ny + 1
    return coords[0] + NI * (coords[1] + NJ_ * coords[2])


def _order_entities(keys_unique: np.ndarray, mesh: StructuredMesh) -> np.ndarray:
    """Sort lattice keys by (entity dimension, key)."""
    nx, ny, nz = mesh.shape
    NI, NJ_ = 2 * nx + 1, 2 * ny + 1
    I = keys_unique % NI
    J = (keys_unique // NI) % NJ_
    K = keys_unique // (NI * NJ_)
    dim = (I % 2) + (J % 2) + (K % 2)
    return keys_unique[np.lexsort((keys_unique, dim))]


def build_dofmap(mesh: StructuredMesh, u_dirichlet_tags: Sequence[str], j_dirichlet_tags: Sequence[str],
                 u_values: Optional[Callable[[np.ndarray, np.ndarray], np.ndarray]] = None) -> DofMap:
    """Number the dofs of the four fields on ``mesh``.

    ``u_values(points, tag_of_point)`` returns the Dirichlet velocity (n,3) at
    the given Dirichlet lattice points (default zero), mirroring the
    ``params[:bcs][:u][:values]`` interpolation (src/fespaces.jl:48-61)."""
    ijk = mesh.cells()
    nc = len(ijk)
    nx, ny, nz = mesh.shape
    # --------------------------------------------------------------- u (Q2 lattice)
    a = np.arange(3)
    la, lb, lc = np.meshgrid(a, a, a, indexing="ij")  # local node n = a + 3b + 9c
    la, lb, lc = la.transpose(2, 1, 0).ravel(), lb.transpose(2, 1, 0).ravel(), lc.transpose(2, 1, 0).ravel()
    I = 2 * ijk[:, 0:1] + la[None, :]
    J = 2 * ijk[:, 1:2] + lb[None, :]
    K = 2 * ijk[:, 2:3] + lc[None, :]
    ukeys = _lattice_keys(mesh, I, J, K)                     # (nc, 27)
    uniq = np.unique(ukeys)
    order = _order_entities(uniq, mesh)
    # Dirichlet lattice points: the 3x3 lattice points of each Dirichlet boundary face
    bcell, bface, btag = mesh.boundary_faces()
    utags = set(mesh.tag_index(u_dirichlet_tags))
    jtags = set(mesh.tag_index(j_dirichlet_tags))
    dmask_u = np.isin(btag, list(utags)) if utags else np.zeros(len(btag), bool)
    dir_keys = []
    for f in range(6):
        sel = np.nonzero(dmask_u & (bface == f))[0]
        if len(sel) == 0:
            continue
        ax, side = FACE_AXIS[f], FACE_SIDE[f]
        on = [la, lb, lc][ax] == 2 * side
        dir_keys.append(ukeys[bcell[sel]][:, on].ravel())
    dir_keys = np.unique(np.concatenate(dir_keys)) if dir_keys else np.zeros(0, np.int64)
    is_dir = np.isin(order, dir_keys)
    free_keys, dkeys = order[~is_dir], order[is_dir]
    # map key -> node id (free >= 0, Dirichlet -(id+1))
    key_sorted = np.argsort(order)
    node_id = np.empty(len(order), np.int64)
    node_id[~is_dir] = np.arange(len(free_keys))
    node_id[is_dir] = -(np.arange(len(dkeys)) + 1)
    pos = np.searchsorted(order[key_sorted], ukeys)
    nid = node_id[key_sorted][pos]                          # (nc, 27)
    cell_dofs = np.empty((nc, 129), dtype=np.int64)
    for comp in range(3):
        fr = nid >= 0
        d = np.where(fr, 3 * nid + comp, -(3 * (-nid - 1) + comp) - 1)
        cell_dofs[:, OU + comp * 27:OU + (comp + 1) * 27] = d
    # physical coordinates of lattice points (for Dirichlet values and node output)
    def key_coords(keys):
        NI, NJ_ = 2 * nx + 1, 2 * ny + 1
        Ik, Jk, Kk = keys % NI, (keys // NI) % NJ_, keys // (NI * NJ_)
        # interpolate trilinearly inside the lattice cell (lattice points are on the
        # Q1 geometry: vertices, edge midpoints, face and cell centres)
        i0 = np.minimum(Ik // 2, nx - 1); j0 = np.minimum(Jk // 2, ny - 1); k0 = np.minimum(Kk // 2, nz - 1)
        xi = (Ik - 2 * i0) / 2.0; yi = (Jk - 2 * j0) / 2.0; zi = (Kk - 2 * k0) / 2.0
        P = np.zeros((len(keys), 3))
        for cc in range(2):
            for bb in range(2):
                for aa in range(2):
                    w = (xi if aa else 1 - xi) * (yi if bb else 1 - yi) * (zi if cc else 1 - zi)
                    P += w[:, None] * mesh.nodes[i0 + aa, j0 + bb, k0 + cc]
        return P
    udir = np.zeros(3 * len(dkeys))
    if u_values is not None and len(dkeys):
        vals = np.asarray(u_values(key_coords(dkeys)), dtype=float).reshape(len(dkeys), 3)
        udir = vals.reshape(-1)
    # --------------------------------------------------------------- p, φ (cell-local)
    cell_dofs[:, OP:OP + NP] = 4 * np.arange(nc)[:, None] + np.arange(4)[None, :]
    cell_dofs[:, OPHI:OPHI + NPHI] = 8 * np.arange(nc)[:, None] + np.arange(8)[None, :]
    # --------------------------------------------------------------- j (RT1)
    # face centre lattice keys per local face
    fkeys = np.empty((nc, 6), dtype=np.int64)
    cI, cJ, cK = 2 * ijk[:, 0] + 1, 2 * ijk[:, 1] + 1, 2 * ijk[:, 2] + 1
    for f in range(6):
        ax, side = FACE_AXIS[f], FACE_SIDE[f]
        c = [cI.copy(), cJ.copy(), cK.copy()]
        c[ax] = c[ax] - 1 + 2 * side
        fkeys[:, f] = _lattice_keys(mesh, *c)
    funiq = np.unique(fkeys)
    forder = np.sort(funiq)
    jdir_mask = np.isin(btag, list(jtags)) if jtags else np.zeros(len(btag), bool)
    jdir_keys = np.unique(fkeys[bcell[jdir_mask], bface[jdir_mask]]) if jdir_mask.any() else np.zeros(0, np.int64)
    fdir = np.isin(forder, jdir_keys)
    nff = int((~fdir).sum())
    fid = np.empty(len(forder), np.int64)
    fid[~fdir] = np.arange(nff)
    fid[fdir] = -(np.arange(int(fdir.sum())) + 1)
    fid_cell = fid[np.searchsorted(forder, fkeys)]          # (nc, 6)
    nj_face_free = 4 * nff
    for b in range(36):
        d, q, l = RT_AXIS[b], RT_Q[b], RT_L[b]
        if q == 1:
            interior = nj_face_free + 12 * np.arange(nc) + 4 * d + l
            cell_dofs[:, OJ + b] = interior
        else:
            f = 2 * d + (1 if q == 2 else 0)
            idf = fid_cell[:, f]
            cell_dofs[:, OJ + b] = np.where(idf >= 0, 4 * idf + l, -(4 * (-idf - 1) + l) - 1)
    ndir_j = 4 * int(fdir.sum())
    nfree = dict(u=3 * len(free_keys), p=4 * nc, j=nj_face_free + 12 * nc, phi=8 * nc)
    offsets = dict(u=0, p=nfree["u"], j=nfree["u"] + nfree["p"], phi=nfree["u"] + nfree["p"] + nfree["j"])
    if cell_dofs.max() >= 2 ** 31:
        raise ValueError("dof ids exceed int32")
    return DofMap(ncells=nc, cell_dofs=cell_dofs.astype(np.int32), nfree=nfree,
                  ndir=dict(u=3 * len(dkeys), p=0, j=ndir_j, phi=0),
                  dir_values=dict(u=udir, j=np.zeros(ndir_j)),
                  u_node_coords=key_coords(free_keys), offsets=offsets)


def touched_block_mask() -> np.ndarray:
    """(129,129) bool: local (row, col) pairs inside the blocks the Jacobian touches
    (uu, up, uj, pu, jj, jφ, ju, φj; src/weakforms.jl:311)."""
    f = np.empty(129, dtype=np.int64)
    f[OU:OU + NU] = 0; f[OP:OP + NP] = 1; f[OJ:OJ + NJ] = 2; f[OPHI:OPHI + NPHI] = 3
    touched = {(0, 0), (0, 1), (0, 2), (1, 0), (2, 2), (2, 3), (2, 0), (3, 2)}
    m = np.zeros((129, 129), bool)
    for (a, b) in touched:
        m[np.ix_(f == a, f == b)] = True
    return m
