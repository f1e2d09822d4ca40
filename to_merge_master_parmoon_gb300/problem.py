"""Python view of the host-side Oseen problem builder (libpmhost.so).

An :class:`OseenProblem` owns the multigrid hierarchy that ParMooN's
TSystemNSE3D would hand to its saddle-point solver: per level the NSTYPE-4
CSR matrices (A11..A33 on one pattern, B1..B3, B1T..B3T), the Q2/P1disc cell
DOF maps and the parent/child relation; plus the finest-level right-hand side.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import PmhParams, PmLevelDesc, host_lib

EXAMPLES = {"random": 0, "quadlin_stokes": 1, "quadlin_oseen": 2, "channel": 3}
PERIODIC = {"x": 1, "y": 2, "z": 4}
ELEMENTS = {"hexa": 0, "tetra": 1}


class OseenProblem:
    """Steady Oseen problem on a box with ``n_levels`` uniform refinements.

    The coarsest level has ``(nx0, ny0, nz0)`` hexahedra; level ``l`` has
    ``2**l`` times as many per direction.  ``example`` selects the seeded
    random Oseen problem (divergence-free Fourier convection, smooth forcing,
    u = 0 on the walls) or the known-answer polynomial solution of the
    reference's Examples/NSE_3D/AnsatzQuadLin.h (Stokes, or Oseen with b := u),
    or the channel ("channel": b = u0 = parabola (1 - eta^2) e_x plus a seeded
    divergence-free perturbation of size ``perturb`` vanishing at the y
    walls, the body force that holds the parabola, u = 0 on the y walls).
    ``periodic`` names identified directions ("xz"), ``stretch_y`` > 0 moves the
    y nodes of every level to y0 + Ly (1 + tanh(s eta)/tanh(s))/2.
    ``element="tetra"`` splits every cube into 6 Kuhn tetrahedra with P2 + face
    and cell bubbles / P1disc (15 + 4 local DOFs) and hands the prolongation
    over in the level descriptors (uniform grids, no periodic directions).
    """

    def __init__(self, n_levels: int = 4, nu: float = 1e-2, seed: int = 0,
                 example: str = "random", nx0: int = 2, ny0: int = 2, nz0: int = 2,
                 box=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0), n_modes: int = 8, nthreads: int = 0,
                 periodic: str = "", stretch_y: float = 0.0, perturb: float = 0.05,
                 element: str = "hexa"):
        lib = host_lib()
        p = PmhParams()
        lib.pmh_default_params(C.byref(p))
        p.nx0, p.ny0, p.nz0, p.n_levels = nx0, ny0, nz0, n_levels
        p.x0, p.x1, p.y0, p.y1, p.z0, p.z1 = box
        p.nu = nu
        p.seed = seed
        p.example = EXAMPLES[example]
        p.n_modes = n_modes
        p.nthreads = nthreads
        p.periodic = sum(PERIODIC[c] for c in periodic)
        p.stretch_y = stretch_y
        p.perturb = perturb
        p.element = ELEMENTS[element]
        self._lib = lib
        self.params = p
        self.nu = nu
        self.example = example
        self.element = element
        self._h = lib.pmh_build(C.byref(p))
        if not self._h:
            raise ValueError("pmh_build rejected the parameters (a periodic direction "
                             "needs an even number >= 2 of coarsest cells)")
        self.n_levels = lib.pmh_n_levels(self._h)
        self._descs = (PmLevelDesc * self.n_levels)()
        for level in range(self.n_levels):
            lib.pmh_level_desc(self._h, level, C.byref(self._descs[level]))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.pmh_free(h)
            self._h = None

    @property
    def descs(self):
        """ctypes array of pm_level_desc, coarsest first (valid while self lives)."""
        return self._descs

    def desc(self, level: int) -> PmLevelDesc:
        return self._descs[level]

    def cell_sizes(self, level: int) -> np.ndarray:
        """(hx, hy, hz) of every cell of a level, shape (n_cells, 3)."""
        d = self._descs[level % self.n_levels]
        out = np.empty((d.n_cells, 3))
        if self._lib.pmh_cell_sizes(self._h, level % self.n_levels,
                                    out.ctypes.data_as(C.POINTER(C.c_double))) != 0:
            raise ValueError("bad level")
        return out

    def convection_nodal(self, level: int) -> np.ndarray:
        """The convection field at the level's velocity nodes, [b1|b2|b3]."""
        d = self._descs[level % self.n_levels]
        out = np.empty(3 * d.n_udof)
        if self._lib.pmh_convection_nodal(self._h, level % self.n_levels,
                                          out.ctypes.data_as(C.POINTER(C.c_double))) != 0:
            raise ValueError("bad level")
        return out

    def reassemble(self):
        """Assemble every level's matrix values again on the host (the build's
        cell loop and threads); the arrays behind ``descs`` are rewritten."""
        if self._lib.pmh_reassemble(self._h) != 0:
            raise ValueError("pmh_reassemble failed")

    def is_one_block(self) -> bool:
        """True when every level has A12..A32 = 0 on the active rows and
        A11 = A22 = A33 exactly (the Galerkin Oseen/Stokes forms with the
        gradient Laplacian), i.e. the system is also an NSTYPE-2 system."""
        for level in range(self.n_levels):
            d = self.arrays(level)
            a, nact = d["a"], d["n_active"]
            act = np.repeat(np.arange(d["n_udof"]) < nact, np.diff(d["a_rowptr"]))
            if not (np.array_equal(a[0], a[4]) and np.array_equal(a[0], a[8])):
                return False
            if any(np.any(a[k][act] != 0.0) for k in (1, 2, 3, 5, 6, 7)):
                return False
        return True

    def descs_one_block(self):
        """The same levels as NSTYPE-2 descriptors: a[0] carries the block of
        all three components, a[1..8] are NULL (TNSE_MGLevel2's one A
        matrix).  Valid only when is_one_block(); shares this problem's arrays."""
        if not self.is_one_block():
            raise ValueError("the velocity blocks are coupled or differ: not an NSTYPE-2 system")
        out = (PmLevelDesc * self.n_levels)()
        for level in range(self.n_levels):
            C.pointer(out[level])[0] = self._descs[level]
            for k in range(1, 9):
                out[level].a[k] = None
        return out

    def ndof(self, level: int = -1) -> int:
        level = level % self.n_levels
        return self._lib.pmh_ndof(self._h, level)

    def rhs(self) -> np.ndarray:
        n = self.ndof(-1)
        return np.ctypeslib.as_array(self._lib.pmh_rhs(self._h), shape=(n,)).copy()

    def exact(self):
        ptr = self._lib.pmh_exact(self._h)
        if not ptr:
            return None
        return np.ctypeslib.as_array(ptr, shape=(self.ndof(-1),)).copy()

    def arrays(self, level: int) -> dict:
        """Numpy views of one level's arrays (no copies)."""
        d = self._descs[level % self.n_levels]

        def iv(ptr, n):
            return np.ctypeslib.as_array(ptr, shape=(n,)) if n > 0 and ptr else np.zeros(0, np.int32)

        def dv(ptr, n):
            return np.ctypeslib.as_array(ptr, shape=(n,))

        out = {
            "n_udof": d.n_udof, "n_pdof": d.n_pdof, "n_active": d.n_active,
            "n_cells": d.n_cells,
            "a_rowptr": iv(d.a_rowptr, d.n_udof + 1), "a_col": iv(d.a_col, d.a_nnz),
            "a": [dv(d.a[k], d.a_nnz) for k in range(9)],
            "b_rowptr": iv(d.b_rowptr, d.n_pdof + 1), "b_col": iv(d.b_col, d.b_nnz),
            "b": [dv(d.b[k], d.b_nnz) for k in range(3)],
            "bt_rowptr": iv(d.bt_rowptr, d.n_udof + 1), "bt_col": iv(d.bt_col, d.bt_nnz),
            "bt": [dv(d.bt[k], d.bt_nnz) for k in range(3)],
            "cell_udofs": iv(d.cell_udofs, d.n_ulocal * d.n_cells).reshape(d.n_cells, d.n_ulocal),
            "cell_pdofs": iv(d.cell_pdofs, 4 * d.n_cells).reshape(d.n_cells, 4),
            "cell_colour": iv(d.cell_colour, d.n_cells),
        }
        if d.cell_parent:
            out["cell_parent"] = iv(d.cell_parent, d.n_cells)
        if d.cell_child:
            out["cell_child"] = iv(d.cell_child, d.n_cells)
        if d.pu_rowptr:
            out["pu_rowptr"] = iv(d.pu_rowptr, d.n_udof + 1)
            out["pu_col"] = iv(d.pu_col, d.pu_nnz)
            out["pu_val"] = dv(d.pu_val, d.pu_nnz)
            out["pp_rowptr"] = iv(d.pp_rowptr, d.n_pdof + 1)
            out["pp_col"] = iv(d.pp_col, d.pp_nnz)
            out["pp_val"] = dv(d.pp_val, d.pp_nnz)
        return out

    def scipy_matrix(self, level: int = -1):
        """Assembled saddle-point matrix K of one level as scipy CSR, with the
        reference's conventions (Dirichlet rows: diagonal blocks only; BT on
        active rows only).  Test helper."""
        import scipy.sparse as sp
        a = self.arrays(level)
        nu, np_, na = a["n_udof"], a["n_pdof"], a["n_active"]
        rows = np.repeat(np.arange(nu), np.diff(a["a_rowptr"]))
        cols = a["a_col"]
        blocks = []
        act = rows < na
        for bi in range(3):
            for bj in range(3):
                v = a["a"][3 * bi + bj].copy()
                if bi != bj:
                    v[~act] = 0.0
                blocks.append(sp.csr_matrix((v, (rows + bi * nu, cols + bj * nu)),
                                            shape=(3 * nu + np_, 3 * nu + np_)))
        brow = np.repeat(np.arange(np_), np.diff(a["b_rowptr"]))
        for k in range(3):
            blocks.append(sp.csr_matrix((a["b"][k], (brow + 3 * nu, a["b_col"] + k * nu)),
                                        shape=(3 * nu + np_, 3 * nu + np_)))
        btrow = np.repeat(np.arange(nu), np.diff(a["bt_rowptr"]))
        bact = btrow < na
        for k in range(3):
            v = a["bt"][k].copy()
            v[~bact] = 0.0
            blocks.append(sp.csr_matrix((v, (btrow + k * nu, a["bt_col"] + 3 * nu)),
                                        shape=(3 * nu + np_, 3 * nu + np_)))
        K = blocks[0]
        for b in blocks[1:]:
            K = K + b
        return K.tocsr()
