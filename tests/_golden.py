"""Loads the golden fixtures (tests/golden/*.npz) written by make_golden.py, and the
solver cases on the reference's example grids (tests/golden/examples/*.npz)."""
import glob
import os

import numpy as np

from suntans_gb300.grid import HProblem, QProblem, SolverProps, SunGrid

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fixture_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "*.npz")))


def example_names():
    """Solver cases on the reference's example grids (tests/golden/examples/,
    written by make_example_golden.py)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "examples", "*.npz")))


def load_example(name):
    return _load(os.path.join(HERE, "examples", name + ".npz"), name)


def load(name):
    return _load(os.path.join(HERE, name + ".npz"), name)


def _load(path, name):
    d = dict(np.load(path))
    Nc, Ne, mf, Nkmax = (int(v) for v in d["sizes"])
    g = SunGrid(Nc=Nc, Ne=Ne, maxfaces=mf, Nkmax=Nkmax,
                **{k: d[k] for k in ("nfaces", "neigh", "face", "Nk", "Nke", "ctop", "cellp", "celldist",
                                     "Ac", "df", "dg", "dzz", "dzf")}, name=name)
    qp = QProblem(grid=g, D=d["qD"], src=d["src"], q=d["q0"], c=d["c0"])
    hp = HProblem(grid=g, D=d["hD"], htmp=d["htmp"], h=d["h0"])
    pv = d["props"]
    props = dict(qmaxiters=int(pv[0]), qepsilon=float(pv[1]), resnorm=float(pv[2]), dt=float(pv[3]),
                 theta=float(pv[4]), grav=float(pv[5]), maxiters=int(pv[6]), epsilon=float(pv[7]))
    return g, qp, hp, props, d


def step_fields(g, d):
    """The step fields stored with a fixture (ComputeQSource / Corrector inputs)."""
    import numpy as np
    from suntans_gb300.grid import StepFields
    g.normal, g.grad = d["normal"], d["grad"]
    return StepFields(grid=g, u=d["u"], utmp2=d["utmp2"], w=d["w"], wtmp2=d["wtmp2"], q=d["qtot"],
                      qc=np.zeros(g.n3), c=np.ones(g.n3), etop=d["etop"], edgep=d["edgep"], edgedist=d["edgedist"])


def vgrid_fields(g, d, smoothbot=0.0):
    """The UpdateDZ / SetFluxHeight inputs stored with a fixture."""
    from suntans_gb300.grid import VGridFields
    g.dz, g.dv, g.grad, g.normal = d["vg_dz"], d["vg_dv"], d["grad"], d["normal"]
    return VGridFields(grid=g, h=d["vg_h"], u=d["vg_u"], dzbot=d["vg_dzbot"], Nkc=d["vg_Nkc"], smoothbot=smoothbot,
                       dzsmall=0.1, ctop=d["vg_ctop"], etop=d["vg_etop"], dzz=d["vg_dzz"])


def upred_fields(g, d, nl):
    """The UPredictor inputs stored with a fixture (nl: implicit vertical advection)."""
    from suntans_gb300.grid import UPredFields
    g.dz, g.dv, g.grad, g.normal = d["vg_dz"], d["vg_dv"], d["grad"], d["normal"]
    pre = f"up{nl}_"
    par = d[pre + "par"]
    kw = {k: d[pre + k] for k in ("u", "w", "h", "utmp", "tau_T", "CdT", "CdB", "nu_tv", "nu_lax", "etop", "edgep",
                                  "edgedist", "bedgep", "bedgedist", "mark", "n1", "n2")}
    return UPredFields(grid=g, nu=float(par[0]), laxWendroff_Vertical=float(par[1]), thetaM=float(par[2]),
                       nonlinear=int(par[3]), **kw)


def wpred_fields(g, d, tag):
    """The WPredictor inputs stored with a fixture (tag "wp1_" or "wp0_")."""
    from suntans_gb300.grid import WPredFields
    g.grad, g.normal = d["grad"], d["normal"]
    par = d[tag + "par"]
    kw = {k: d[tag + k] for k in ("w", "Cn_W", "Cn_W2", "q", "nu_tv", "nu_lax", "utmp2")}
    return WPredFields(grid=g, nu=float(par[0]), nu_H=float(par[1]), CdW=float(par[2]),
                       laxWendroff_Vertical=float(par[3]), nonlinear=int(par[4]), conserveMomentum=int(par[5]),
                       n=int(par[6]), AB=int(par[7]), etop=d["etop"], edgep=d["edgep"], edgedist=d["edgedist"],
                       **kw)


def props_for(props, **kw):
    return SolverProps(**{**props, **kw})


LOCKX = os.path.join(HERE, "runs", "lockexchange_cfg1.npz")


def load_lockexchange():
    """The 64 x 16 lock-exchange channel's solver fixture (make_lockexchange_golden.py):
    returns (d, props, grid_at, q_problem, h_problem) where grid_at(step)
    builds the solver grid with that step's ctop/dzz/dzf and the problem
    builders return (problem, reference solution, reference iterations)."""
    d = dict(np.load(LOCKX))
    Nc, Ne, mf, Nkmax = (int(v) for v in d["sizes"])
    pv = d["props"]
    props = SolverProps(qprecond=int(pv[9]), qmaxiters=int(pv[7]), qepsilon=float(pv[4]), hprecond=int(pv[8]),
                        maxiters=int(pv[6]), epsilon=float(pv[3]), resnorm=float(pv[5]), grav=float(pv[2]),
                        theta=float(pv[1]), dt=float(pv[0]))
    base = {k: d[k] for k in ("nfaces", "neigh", "face", "Nk", "Nke", "cellp", "celldist", "Ac", "df", "dg")}
    first_q = int(d["q_steps"][0])

    def grid_at(step):
        qs = step if f"q{step}_ctop" in d else first_q
        return SunGrid(Nc=Nc, Ne=Ne, maxfaces=mf, Nkmax=Nkmax, ctop=d[f"q{qs}_ctop"], dzz=d[f"q{qs}_dzz"],
                       dzf=d[f"q{qs}_dzf"], name=f"lockexchange_step{step}", **base)

    def q_problem(step):
        g = grid_at(step)
        p = QProblem(grid=g, D=d[f"q{step}_D"], src=d[f"q{step}_src"], q=d[f"q{step}_q_in"], c=np.ones(g.n3))
        return p, d[f"q{step}_q_out"], int(d[f"q{step}_niters"][0])

    def h_problem(step):
        g = grid_at(step)
        p = HProblem(grid=g, D=d[f"h{step}_D"], htmp=d[f"h{step}_htmp"], h=d[f"h{step}_h_in"])
        return p, d[f"h{step}_h_out"], int(d[f"h{step}_niters"][0])

    return d, props, grid_at, q_problem, h_problem
