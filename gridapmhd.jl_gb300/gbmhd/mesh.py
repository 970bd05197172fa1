"""Structured hexahedral meshes for the Hunt duct and the sudden expansion.

Host-side mirror of the reference meshers:

* ``hunt_generate_base_mesh`` (GridapMHD src/Meshers/hunt_mesher.jl:109-138):
  a ``CartesianDiscreteModel`` over ``(-1,1,-1,1,0,Lz)`` with ``nz`` axial cells,
  periodic in z, whose node coordinates are passed through a map.
* ``strechMHD`` / ``hunt_stretch_map`` (src/Meshers/hunt_mesher.jl:5-46): the
  Smolentsev boundary-layer map and the power-law map, plus the tanh map
  ``x -> tanh(b x)/tanh(b)`` used by the GPU benchmark configurations.
* ``hunt_add_tags!`` (src/Meshers/hunt_mesher.jl:54-102): walls y=±1 are
  "conducting" (Hartmann walls, B along y), walls x=±1 are "insulating",
  every wall is "noslip".
* The sudden expansion (src/Applications/expansion.jl:267-381 semantics) as a
  structured box grid with the step region removed.

A mesh is a tensor grid of (nx, ny, nz) cells, an ``active`` cell mask, node
coordinates of the mapped lattice (not glued, so periodic cells keep their
true geometry), and periodicity flags.  Cells are ordered lexicographically
with x fastest, like ``CartesianDiscreteModel``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

# Local faces of a cell: index = axis*2 + side, side 0 is the lower face.
FACE_AXIS = np.array([0, 0, 1, 1, 2, 2])
FACE_SIDE = np.array([0, 1, 0, 1, 0, 1])


@dataclass
class StructuredMesh:
    """Tensor-grid hexahedral mesh (see module docstring)."""

    nodes: np.ndarray                 # (nx+1, ny+1, nz+1, 3) mapped lattice coordinates
    active: np.ndarray                # (nx, ny, nz) bool
    periodic: Tuple[bool, bool, bool]
    face_classifier: Callable[[np.ndarray, np.ndarray], np.ndarray]
    tag_names: List[str]
    name: str = "mesh"
    meta: Dict = field(default_factory=dict)

    @property
    def shape(self) -> Tuple[int, int, int]:
        return tuple(int(s) for s in self.active.shape)  # type: ignore[return-value]

    def cells(self) -> np.ndarray:
        """(ncells, 3) integer (i, j, k) of active cells, x fastest."""
        nx, ny, nz = self.shape
        k, j, i = np.nonzero(np.transpose(self.active, (2, 1, 0)))
        return np.stack([i, j, k], axis=1).astype(np.int64)

    @property
    def ncells(self) -> int:
        return int(self.active.sum())

    def cell_coords(self) -> np.ndarray:
        """(ncells, 8, 3) vertex coordinates, local vertex a + 2b + 4c."""
        ijk = self.cells()
        out = np.empty((len(ijk), 8, 3))
        for c in range(2):
            for b in range(2):
                for a in range(2):
                    out[:, a + 2 * b + 4 * c, :] = self.nodes[ijk[:, 0] + a, ijk[:, 1] + b, ijk[:, 2] + c]
        return out

    def boundary_faces(self) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        """Faces of active cells with no active neighbour across them.

        Returns (cell index into cells(), local face 0..5, tag index)."""
        nx, ny, nz = self.shape
        ijk = self.cells()
        dims = np.array([nx, ny, nz])
        cell_ids, lfaces = [], []
        for f in range(6):
            ax, side = FACE_AXIS[f], FACE_SIDE[f]
            nb = ijk.copy()
            nb[:, ax] += 1 if side else -1
            if self.periodic[ax]:
                nb[:, ax] %= dims[ax]
                inside = np.ones(len(ijk), bool)
            else:
                inside = (nb[:, ax] >= 0) & (nb[:, ax] < dims[ax])
            nbc = np.clip(nb, 0, dims - 1)
            nb_active = inside & self.active[nbc[:, 0], nbc[:, 1], nbc[:, 2]]
            sel = np.nonzero(~nb_active)[0]
            cell_ids.append(sel)
            lfaces.append(np.full(len(sel), f))
        cell_ids = np.concatenate(cell_ids)
        lfaces = np.concatenate(lfaces)
        order = np.lexsort((lfaces, cell_ids))
        cell_ids, lfaces = cell_ids[order], lfaces[order]
        centers = self.face_centers(cell_ids, lfaces)
        normals = np.zeros((len(cell_ids), 3))
        normals[np.arange(len(cell_ids)), FACE_AXIS[lfaces]] = np.where(FACE_SIDE[lfaces] == 1, 1.0, -1.0)
        tags = self.face_classifier(centers, normals)
        return cell_ids.astype(np.int64), lfaces.astype(np.int64), tags.astype(np.int64)

    def face_centers(self, cell_ids: np.ndarray, lfaces: np.ndarray) -> np.ndarray:
        ijk = self.cells()[cell_ids]
        ax, side = FACE_AXIS[lfaces], FACE_SIDE[lfaces]
        pts = np.zeros((len(cell_ids), 3))
        cnt = 0
        for c in range(2):
            for b in range(2):
                for a in range(2):
                    off = np.stack([np.full(len(ijk), a), np.full(len(ijk), b), np.full(len(ijk), c)], 1)
                    on_face = off[np.arange(len(ijk)), ax] == side
                    p = self.nodes[ijk[:, 0] + a, ijk[:, 1] + b, ijk[:, 2] + c]
                    pts += np.where(on_face[:, None], p, 0.0)
                    cnt += 1
        return pts / 4.0

    def tag_index(self, names: Sequence[str]) -> List[int]:
        out = []
        for n in names:
            if n not in self.tag_names:
                raise KeyError(f"unknown boundary tag {n!r}; mesh has {self.tag_names}")
            out.append(self.tag_names.index(n))
        return out


# ----------------------------------------------------------------------- maps

def strech_mhd(x: np.ndarray, xi0: float, xi1: float, factor: float) -> np.ndarray:
    """Smolentsev stretching of one coordinate (src/Meshers/hunt_mesher.jl:5-28)."""
    l = xi1 - xi0
    c = (factor + 1.0) / (factor - 1.0)
    out = np.array(x, dtype=float, copy=True)
    if l > 0:
        m = (xi0 <= x) & (x <= xi1)
    else:
        m = (xi1 <= x) & (x <= xi0)
    xx = (x[m] - xi0) / l
    out[m] = factor * (c ** xx - 1.0) / (1.0 + c ** xx) * l + xi0
    return out


def hunt_stretch_map(L: float, Ha: float, kmap_x: float = 1, kmap_y: float = 1,
                     BL_adapted: bool = True) -> Callable[[np.ndarray], np.ndarray]:
    """Coordinate map of the Hunt mesher (src/Meshers/hunt_mesher.jl:30-46)."""
    if BL_adapted:
        s_ha = math.sqrt(Ha / (Ha - 1.0))
        s_side = math.sqrt(math.sqrt(Ha) / (math.sqrt(Ha) - 1.0))

        def map1(P):
            P = np.array(P, dtype=float, copy=True)
            # first call: domain (0,-L,0,-L); second call on its output: (0,L,0,L)
            P[..., 0] = strech_mhd(P[..., 0], 0.0, -L, s_side)
            P[..., 1] = strech_mhd(P[..., 1], 0.0, -L, s_ha)
            P[..., 0] = strech_mhd(P[..., 0], 0.0, L, s_side)
            P[..., 1] = strech_mhd(P[..., 1], 0.0, L, s_ha)
            return P
        return map1

    def map2(P):
        P = np.array(P, dtype=float, copy=True)
        P[..., 0] = np.sign(P[..., 0]) * np.abs(L * P[..., 0]) ** (1.0 / kmap_x)
        P[..., 1] = np.sign(P[..., 1]) * np.abs(L * P[..., 1]) ** (1.0 / kmap_y)
        return P
    return map2


def tanh_map(beta: float) -> Callable[[np.ndarray], np.ndarray]:
    """x -> tanh(βx)/tanh(β) on the two cross-section coordinates (β=0: identity)."""
    def m(P):
        P = np.array(P, dtype=float, copy=True)
        if beta != 0.0:
            for d in (0, 1):
                P[..., d] = np.tanh(beta * P[..., d]) / math.tanh(beta)
        return P
    return m


# ----------------------------------------------------------------------- Hunt

HUNT_TAGS = ["conducting", "insulating", "z_periodic"]


def _hunt_classifier(centers: np.ndarray, normals: np.ndarray) -> np.ndarray:
    # y-normal walls (Hartmann walls) -> conducting (0); x-normal walls -> insulating (1)
    tags = np.full(len(centers), 2)
    tags[np.abs(normals[:, 1]) > 0.5] = 0
    tags[np.abs(normals[:, 0]) > 0.5] = 1
    return tags


def cartesian_mesh(domain: Sequence[float], partition: Sequence[int],
                   periodic=(False, False, False), map: Optional[Callable] = None,
                   classifier=_hunt_classifier, tag_names=HUNT_TAGS, name="cartesian") -> StructuredMesh:
    """``CartesianDiscreteModel(domain, partition; isperiodic, map)`` restated."""
    nx, ny, nz = (int(p) for p in partition)
    x = np.linspace(domain[0], domain[1], nx + 1)
    y = np.linspace(domain[2], domain[3], ny + 1)
    z = np.linspace(domain[4], domain[5], nz + 1)
    P = np.stack(np.meshgrid(x, y, z, indexing="ij"), axis=-1)
    if map is not None:
        P = map(P)
    return StructuredMesh(nodes=np.ascontiguousarray(P), active=np.ones((nx, ny, nz), bool),
                          periodic=tuple(bool(p) for p in periodic), face_classifier=classifier,
                          tag_names=list(tag_names), name=name)


def hunt_generate_base_mesh(nc: Sequence[int], L: float = 1.0, tw: float = 0.0, Ha: float = 10.0,
                            kmap_x=1, kmap_y=1, BL_adapted=True, nz: int = 3, Lz: float = 0.1,
                            map: Optional[Callable] = None) -> StructuredMesh:
    """Serial Hunt base mesh (src/Meshers/hunt_mesher.jl:125-138).

    The reference hard-codes 3 axial cells over z in (0, 0.1); ``nz``, ``Lz`` and
    ``map`` generalise that for the duct configurations of the GPU benchmark."""
    if tw > 0.0:
        raise NotImplementedError("resolved solid walls (tw>0) are not part of this hot path")
    cmap = map if map is not None else hunt_stretch_map(L + tw, Ha, kmap_x, kmap_y, BL_adapted)
    m = cartesian_mesh((-1.0, 1.0, -1.0, 1.0, 0.0, Lz), (nc[0], nc[1], nz), (False, False, True), cmap,
                       name=f"hunt{nc[0]}x{nc[1]}x{nz}")
    m.meta.update(dict(kind="hunt", nc=tuple(nc), nz=nz, Lz=Lz))
    return m


# ----------------------------------------------------------------------- expansion

EXPANSION_TAGS = ["wall", "inlet", "outlet"]


def graded_points(a: float, b: float, n: int, ratio_a: float = 1.0, ratio_b: float = 1.0) -> np.ndarray:
    """n+1 points on [a,b] clustered toward both ends with a tanh law (ratio ≥ 1)."""
    t = np.linspace(-1.0, 1.0, n + 1)
    s = max(ratio_a, ratio_b)
    if s <= 1.0:
        return np.linspace(a, b, n + 1)
    beta = math.log(s) + 1e-12
    u = np.tanh(beta * t) / math.tanh(beta)
    if ratio_a != ratio_b:
        # one-sided: keep clustering only on the side with the larger ratio
        u = np.where(t < 0, u if ratio_a >= ratio_b else t, u if ratio_b >= ratio_a else t)
    return a + (b - a) * 0.5 * (u + 1.0)


def expansion_mesh(n_up: int = 20, n_down: int = 80, n_y_in: int = 10, n_y_out: int = 20, n_z: int = 10,
                   L_up: float = 2.0, L_down: float = 8.0, h_in: float = 0.5, ratio: float = 4.0,
                   width: float = 1.0, grading: float = 4.0) -> StructuredMesh:
    """Structured sudden expansion (B along y): inlet channel x∈(-L_up,0) of height
    h_in centred on y=0, expanding by ``ratio`` in y at x=0, outlet at x=L_down.

    The y lines are shared by both channels: ``n_y_in`` cells cover the inlet
    height and ``n_y_out`` cells cover each of the two step regions.  Points
    are clustered toward the walls and toward the step plane x=0."""
    H = h_in * ratio
    xs = np.concatenate([graded_points(-L_up, 0.0, n_up, 1.0, grading)[:-1],
                         graded_points(0.0, L_down, n_down, grading, 1.0)])
    y_in = graded_points(-0.5 * h_in, 0.5 * h_in, n_y_in, grading, grading)
    y_lo = graded_points(-0.5 * H, -0.5 * h_in, n_y_out, grading, grading)
    y_hi = graded_points(0.5 * h_in, 0.5 * H, n_y_out, grading, grading)
    ys = np.concatenate([y_lo[:-1], y_in[:-1], y_hi])
    zs = graded_points(-0.5 * width, 0.5 * width, n_z, grading, grading)
    P = np.stack(np.meshgrid(xs, ys, zs, indexing="ij"), axis=-1)
    nx, ny, nz = len(xs) - 1, len(ys) - 1, len(zs) - 1
    active = np.ones((nx, ny, nz), bool)
    xc = 0.5 * (xs[:-1] + xs[1:])
    yc = 0.5 * (ys[:-1] + ys[1:])
    step = (xc[:, None] < 0.0) & (np.abs(yc)[None, :] > 0.5 * h_in)
    active[step, :] = False

    def classifier(centers, normals):
        tags = np.zeros(len(centers), dtype=np.int64)            # wall
        tol = 1e-9
        tags[(np.abs(normals[:, 0]) > 0.5) & (centers[:, 0] < -L_up + tol)] = 1   # inlet
        tags[(np.abs(normals[:, 0]) > 0.5) & (centers[:, 0] > L_down - tol)] = 2  # outlet
        return tags

    m = StructuredMesh(nodes=np.ascontiguousarray(P), active=active, periodic=(False, False, False),
                       face_classifier=classifier, tag_names=list(EXPANSION_TAGS), name="expansion")
    m.meta.update(dict(kind="expansion", L_up=L_up, L_down=L_down, h_in=h_in, H=H, width=width))
    return m
