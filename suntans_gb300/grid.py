"""Host-side description of a SUNTANS grid and of the per-solve fields.

`SunGrid` holds the subset of the reference's `gridT` (main/grid.h:32-149)
that the two elliptic solves read: connectivity (`nfaces`, `neigh`, `face`),
vertical structure (`Nk`, `Nke`, `ctop`, `dzz`, `dzf`), geometry (`Ac`, `df`,
`dg`) and the computational / type-3 boundary cell split (`cellp`,
`celldist`, main/grid.c:1652-1664).  Ragged per-cell arrays (`dzz`, and the
solution / right-hand side of the pressure solve) are stored flat: cell ``i``
occupies ``[coff[i], coff[i] + Nk[i])`` where ``coff`` is the exclusive prefix
sum of ``Nk`` in cell-index order -- the reference's jagged ``REAL **`` rows laid
end to end.  ``dzf`` is flat per edge the same way with ``eoff`` over ``Nke``.
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np

I32 = np.int32
F64 = np.float64


@dataclasses.dataclass
class SunGrid:
    Nc: int
    Ne: int
    maxfaces: int
    Nkmax: int
    nfaces: np.ndarray      # [Nc] int32
    neigh: np.ndarray       # [Nc*maxfaces] int32, -1 = none
    face: np.ndarray        # [Nc*maxfaces] int32
    Nk: np.ndarray          # [Nc] int32
    Nke: np.ndarray         # [Ne] int32
    ctop: np.ndarray        # [Nc] int32
    cellp: np.ndarray       # [Nc] int32
    celldist: np.ndarray    # [3] int32
    Ac: np.ndarray          # [Nc] f64
    df: np.ndarray          # [Ne] f64
    dg: np.ndarray          # [Ne] f64
    dzz: np.ndarray         # ragged per cell, f64
    dzf: np.ndarray         # ragged per edge, f64
    # geometry kept for building right-hand sides (not read by the solvers)
    normal: Optional[np.ndarray] = None   # [Nc*maxfaces] int32, +1 outward along edge normal
    grad: Optional[np.ndarray] = None     # [2*Ne] int32
    xv: Optional[np.ndarray] = None
    yv: Optional[np.ndarray] = None
    dz: Optional[np.ndarray] = None       # [Nkmax] layer thicknesses (gridT.dz)
    dv: Optional[np.ndarray] = None       # [Nc] depth (gridT.dv)
    # plan-view geometry for the grid files (gridT.xp/yp/cells/edges/mark)
    xp: Optional[np.ndarray] = None       # [Np] node coordinates
    yp: Optional[np.ndarray] = None
    cnodes: Optional[np.ndarray] = None   # [Nc*maxfaces] node ids of each cell, -1 pad
    enodes: Optional[np.ndarray] = None   # [2*Ne] node ids of each edge
    mark: Optional[np.ndarray] = None     # [Ne] 0 interior, 1 closed, 3 open (type-3) boundary
    name: str = "grid"

    def __post_init__(self):
        for f in ("nfaces", "neigh", "face", "Nk", "Nke", "ctop", "cellp", "celldist"):
            setattr(self, f, np.ascontiguousarray(getattr(self, f), dtype=I32))
        for f in ("Ac", "df", "dg", "dzz", "dzf"):
            setattr(self, f, np.ascontiguousarray(getattr(self, f), dtype=F64))

    # ---- ragged offsets ----
    @property
    def coff(self) -> np.ndarray:
        o = np.zeros(self.Nc + 1, dtype=np.int64)
        np.cumsum(self.Nk, out=o[1:])
        return o

    @property
    def eoff(self) -> np.ndarray:
        o = np.zeros(self.Ne + 1, dtype=np.int64)
        np.cumsum(self.Nke, out=o[1:])
        return o

    @property
    def n3(self) -> int:
        return int(self.Nk.sum())

    @property
    def ncomp(self) -> int:
        return int(self.celldist[1] - self.celldist[0])

    def comp_cells(self) -> np.ndarray:
        return self.cellp[self.celldist[0]:self.celldist[1]]

    def n_q(self) -> int:
        """Pressure unknowns: sum over computational cells of Nk - ctop."""
        c = self.comp_cells()
        return int((self.Nk[c] - self.ctop[c]).sum())

    def n_h(self) -> int:
        return self.ncomp

    def active_mask(self) -> np.ndarray:
        """Boolean mask over the flat ragged storage: computational cell and k >= ctop."""
        m = np.zeros(self.n3, dtype=bool)
        coff = self.coff
        for i in self.comp_cells():
            m[coff[i] + self.ctop[i]:coff[i + 1]] = True
        return m

    def validate(self) -> None:
        """Host-side index checks run before any upload (raises ValueError)."""
        Nc, Ne, mf = self.Nc, self.Ne, self.maxfaces
        if self.neigh.size != Nc * mf or self.face.size != Nc * mf:
            raise ValueError("neigh/face must have Nc*maxfaces entries")
        if np.any(self.nfaces < 1) or np.any(self.nfaces > mf):
            raise ValueError("nfaces out of [1, maxfaces]")
        if np.any(self.Nk < 1) or np.any(self.Nk > self.Nkmax):
            raise ValueError("Nk out of [1, Nkmax]")
        if np.any(self.ctop < 0) or np.any(self.ctop >= self.Nk):
            raise ValueError("ctop out of [0, Nk)")
        f = np.arange(mf)[None, :] < self.nfaces[:, None]
        nb = self.neigh.reshape(Nc, mf)[f]
        fc = self.face.reshape(Nc, mf)[f]
        if np.any((nb < -1) | (nb >= Nc)):
            raise ValueError("neigh index out of range")
        if np.any((fc < 0) | (fc >= Ne)):
            raise ValueError("face index out of range")
        cells = np.repeat(np.arange(Nc), self.nfaces)
        has = nb >= 0
        if np.any(self.Nke[fc[has]] > np.minimum(self.Nk[cells[has]], self.Nk[nb[has]])):
            raise ValueError("Nke exceeds the Nk of a cell on the edge")
        if self.dzz.size != self.n3 or self.dzf.size != int(self.Nke.sum()):
            raise ValueError("dzz/dzf sizes do not match Nk/Nke")
        cd = self.celldist
        if not (0 == cd[0] <= cd[1] <= cd[2] <= Nc):
            raise ValueError("celldist must be 0 <= c1 <= c2 <= Nc")

    # ---- ragged helpers ----
    def ragged_zeros(self) -> np.ndarray:
        return np.zeros(self.n3, dtype=F64)

    def nbytes(self) -> int:
        return sum(getattr(self, f).nbytes for f in
                   ("nfaces", "neigh", "face", "Nk", "Nke", "ctop", "cellp", "Ac", "df", "dg", "dzz", "dzf"))


@dataclasses.dataclass
class QProblem:
    """Inputs of one pressure solve (CGSolveQ): D, right-hand side, warm start, c."""
    grid: SunGrid
    D: np.ndarray     # [Ne] df/dg (set by ComputeQSource, main/phys.c:2392-2394)
    src: np.ndarray   # ragged: right-hand side (destroyed by the reference)
    q: np.ndarray     # ragged: initial guess in, solution out
    c: np.ndarray     # ragged: preconditioner buffer (read only at type-3 cells)


@dataclasses.dataclass
class HProblem:
    """Inputs of one free-surface solve (CGSolve)."""
    grid: SunGrid
    D: np.ndarray     # [Ne] sum_k E*dzf (UPredictor, main/phys.c:2935-2937)
    htmp: np.ndarray  # [Nc] right-hand side (destroyed by the reference)
    h: np.ndarray     # [Nc] boundary values at type-3 cells; solution out


@dataclasses.dataclass
class StepFields:
    """Fields of the nonhydrostatic pressure step around CGSolveQ (Solve,
    main/phys.c:1273-1287): ComputeQSource reads u*, w* and their previous
    values, Corrector updates u, w and the pressure q with the correction qc."""
    grid: SunGrid
    u: np.ndarray         # ragged per edge (Nke levels): predicted horizontal velocity, corrected in place
    utmp2: np.ndarray     # ragged per edge: the previous step's u (theta-method term)
    w: np.ndarray         # ragged per cell with Nk+1 levels: predicted vertical velocity, corrected in place
    wtmp2: np.ndarray     # ragged per cell with Nk+1 levels: the previous step's w
    q: np.ndarray         # ragged per cell: total nonhydrostatic pressure, += qc
    qc: np.ndarray        # ragged per cell: pressure correction (warm start in, solution out)
    c: np.ndarray         # ragged per cell: CGSolveQ's preconditioner buffer (read at type-3 cells)
    etop: np.ndarray      # [Ne] top wet level of each edge
    edgep: np.ndarray     # computational edges
    edgedist: np.ndarray  # [2]: edgep[edgedist[0]:edgedist[1]]

    @property
    def woff(self) -> np.ndarray:
        o = np.zeros(self.grid.Nc + 1, dtype=np.int64)
        np.cumsum(self.grid.Nk + 1, out=o[1:])
        return o


@dataclasses.dataclass
class VGridFields:
    """Inputs of UpdateDZ and SetFluxHeight beyond the grid: the free surface,
    the edge velocity, the gridT vertical-grid settings and the per-step
    ctop / etop / dzz they start from."""
    grid: SunGrid
    h: np.ndarray         # [Nc] free surface
    u: np.ndarray         # ragged per edge (Nke levels)
    dzbot: np.ndarray     # [Nc] gridT.dzbot
    Nkc: np.ndarray       # [Ne] levels stored per dzf row
    smoothbot: float
    dzsmall: float
    ctop: np.ndarray      # [Nc] current ctop
    etop: np.ndarray      # [Ne] current etop
    dzz: np.ndarray       # ragged per cell: current dzz

    @property
    def foff(self) -> np.ndarray:
        o = np.zeros(self.grid.Ne + 1, dtype=np.int64)
        np.cumsum(self.Nkc, out=o[1:])
        return o


@dataclasses.dataclass
class UPredFields:
    """Inputs of UPredictor (main/phys.c:2579-3077) beyond the grid: the state
    at step n, the explicit horizontal source, the drag and viscosity fields,
    and the edge orderings (computational edges, and all edges by mark as
    main/grid.c:1666-1679 orders them)."""
    grid: SunGrid
    u: np.ndarray         # ragged per edge (Nke levels): u at step n
    w: np.ndarray         # ragged per cell (Nk+1 levels): w at step n
    h: np.ndarray         # [Nc] free surface at step n
    utmp: np.ndarray      # ragged per edge: explicit horizontal source in, U*** out
    tau_T: np.ndarray     # [Ne] surface stress
    CdT: np.ndarray       # [Ne] top drag coefficient (-1 = no slip)
    CdB: np.ndarray       # [Ne] bottom drag coefficient (-1 = no slip)
    nu_tv: np.ndarray     # ragged per cell: vertical eddy viscosity
    nu_lax: np.ndarray    # ragged per cell: Lax-Wendroff viscosity
    nu: float
    laxWendroff_Vertical: float
    thetaM: float         # < 0: no implicit vertical momentum advection
    nonlinear: int
    etop: np.ndarray      # [Ne] top wet level of each edge
    edgep: np.ndarray     # computational edges
    edgedist: np.ndarray  # [2]
    bedgep: np.ndarray    # all edges ordered by mark
    bedgedist: np.ndarray # [6]
    mark: np.ndarray      # [Ne]
    n1: np.ndarray        # [Ne] unit normal, grad[0] towards grad[1]
    n2: np.ndarray

    @property
    def woff(self) -> np.ndarray:
        o = np.zeros(self.grid.Nc + 1, dtype=np.int64)
        np.cumsum(self.grid.Nk + 1, out=o[1:])
        return o


@dataclasses.dataclass
class WPredFields:
    """Inputs of WPredictor (main/phys.c:2025-2287) beyond the grid: w and its
    Adams-Bashforth histories, the pressure, the viscosities, the advecting face
    velocity and the propT settings it reads."""
    grid: SunGrid
    w: np.ndarray         # ragged per cell (Nk+1 levels)
    Cn_W: np.ndarray      # ragged per cell (Nk levels)
    Cn_W2: np.ndarray     # ragged per cell (Nk levels)
    q: np.ndarray         # ragged per cell: nonhydrostatic pressure
    nu_tv: np.ndarray
    nu_lax: np.ndarray
    utmp2: np.ndarray     # ragged per edge (Nke levels): advecting velocity
    nu: float
    nu_H: float
    CdW: float
    laxWendroff_Vertical: float
    nonlinear: int        # 0 or 1
    conserveMomentum: int
    n: int                # time step index (1: first step)
    AB: int               # 2 or 3
    etop: np.ndarray      # [Ne]
    edgep: np.ndarray     # computational edges
    edgedist: np.ndarray  # [2]

    @property
    def woff(self) -> np.ndarray:
        o = np.zeros(self.grid.Nc + 1, dtype=np.int64)
        np.cumsum(self.grid.Nk + 1, out=o[1:])
        return o


@dataclasses.dataclass
class SolverProps:
    """The propT fields the two solves read (main/phys.h:183-203)."""
    qprecond: int = 1
    qmaxiters: int = 1000
    qepsilon: float = 1e-10
    hprecond: int = 1
    maxiters: int = 1000
    epsilon: float = 1e-10
    resnorm: float = 1.0
    grav: float = 9.81
    theta: float = 0.55
    dt: float = 1.0
