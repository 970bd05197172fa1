"""Workloads of the benchmark configurations and the tests: Hunt ducts in the CFD scaling
(src/Applications/hunt.jl:95-193) and the sudden expansion in the MHD scaling
(src/Applications/expansion.jl:109-192), as (mesh, dof map, parameters), and a GPU context
built from them through the C ABI."""
import numpy as np

from .fespace import build_dofmap
from .mesh import hunt_generate_base_mesh, tanh_map


def hunt_case(nc=(4, 4), nz=3, Ha=10.0, Re=10.0, beta_map=0.0, Lz=0.1, cw=0.0, tau=100.0, perturb=0.0,
              convection=2, zeta_u=0.0, zeta_j=0.0, f=(0.0, 0.0, 1.0), f_cell=None, seed=0, Bdir=(0, 1, 0)):
    """Hunt duct in CFD scaling (α=1, β=1/Re, γ=Ha²/Re): conducting (or thin-wall) Hartmann
    walls y=±1, insulating side walls x=±1, no-slip everywhere, periodic in z."""
    if perturb > 0.0:
        rng = np.random.default_rng(seed)

        def m(P):
            P = tanh_map(beta_map)(P)
            d = rng.uniform(-perturb, perturb, P.shape)
            h = 2.0 / max(nc)
            inner = (np.abs(P[..., 0]) < 1 - 1e-9) & (np.abs(P[..., 1]) < 1 - 1e-9)
            d[..., 2] = 0.0
            return P + np.where(inner[..., None], d * h, 0.0)
        mesh = hunt_generate_base_mesh(nc, Ha=Ha, nz=nz, Lz=Lz, map=m)
    else:
        mesh = hunt_generate_base_mesh(nc, Ha=Ha, nz=nz, Lz=Lz, map=tanh_map(beta_map))
    dm = build_dofmap(mesh, ["conducting", "insulating"], ["insulating"])
    params = dict(alpha=1.0, beta=1.0 / Re, gamma=Ha ** 2 / Re, sigma=1.0, B=Bdir, f=f, zeta_u=zeta_u,
                  zeta_j=zeta_j, convection=convection)
    facets = None
    if cw > 0:
        bc, bf, bt = mesh.boundary_faces()
        sel = bt == mesh.tag_names.index("conducting")
        n = int(sel.sum())
        facets = dict(cell=bc[sel].astype(np.int32), lface=bf[sel].astype(np.int8), tau=np.full(n, tau),
                      cw=np.full(n, cw), jw=np.zeros(n), phi0=None)
    if f_cell is not None:
        params["f_cell"] = f_cell
    params["facets"] = facets
    return mesh, dm, params


def gpu_context(mesh, dm, params):
    from .lib import Context
    return Context(mesh.cell_coords(), dm.cell_dofs, [dm.nfree[f] for f in ("u", "p", "j", "phi")],
                   [dm.ndir[f] for f in ("u", "p", "j", "phi")],
                   [dm.dir_values.get(f) for f in ("u", "p", "j", "phi")], params)


def expansion_case(n_up=3, n_down=6, n_y_in=3, n_y_out=3, n_z=3, Ha=20.0, Re=10.0, ratio=4.0, convection=2,
                   L_up=1.0, L_down=2.0, grading=2.0, thin_wall=None):
    """Sudden expansion in MHD scaling (α=1/N, β=1/Ha², γ=1; src/Applications/expansion.jl:113-123):
    parabolic inlet velocity, u Dirichlet on walls/inlet, natural (∇p-free) outlet for u,
    B=(0,1,0).  Walls: j Dirichlet on wall, inlet and outlet (insulating, :150-159), or with
    thin_wall=(τ, cw) the thin-wall law on "wall" and j Dirichlet on inlet and outlet only
    (:160-167)."""
    from .mesh import expansion_mesh
    mesh = expansion_mesh(n_up=n_up, n_down=n_down, n_y_in=n_y_in, n_y_out=n_y_out, n_z=n_z, ratio=ratio,
                          L_up=L_up, L_down=L_down, grading=grading)
    h = mesh.meta["h_in"]
    w = mesh.meta["width"]
    H = mesh.meta["H"]

    def u_in(P, *_):
        # parabolic in y and z over the inlet section; mean 1 over the outlet section (flux matching)
        y = P[:, 1] / (0.5 * h)
        z = P[:, 2] / (0.5 * w)
        prof = np.clip((1 - y ** 2) * (1 - z ** 2), 0.0, None)
        scale = (H / h) * (9.0 / 4.0)  # mean of (1-y²)(1-z²) is 4/9; flux = H*w over the outlet
        out = np.zeros((len(P), 3))
        inlet = P[:, 0] < -mesh.meta["L_up"] + 1e-9
        out[inlet, 0] = scale * prof[inlet]
        return out
    jtags = ["wall", "inlet", "outlet"] if thin_wall is None else ["inlet", "outlet"]
    dm = build_dofmap(mesh, ["wall", "inlet"], jtags, u_values=u_in)
    N = Ha ** 2 / Re
    params = dict(alpha=1.0 / N, beta=1.0 / Ha ** 2, gamma=1.0, sigma=1.0, B=(0, 1, 0), f=(0.0, 0.0, 0.0),
                  zeta_u=0.0, zeta_j=0.0, convection=convection, facets=None)
    if thin_wall is not None:
        tau, cw = thin_wall
        bc, bf, bt = mesh.boundary_faces()
        sel = bt == mesh.tag_names.index("wall")
        n = int(sel.sum())
        params["facets"] = dict(cell=bc[sel].astype(np.int32), lface=bf[sel].astype(np.int8), tau=np.full(n, tau),
                                cw=np.full(n, cw), jw=np.zeros(n), phi0=None)
    return mesh, dm, params
