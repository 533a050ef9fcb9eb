"""Command-line drivers that read goal's input files unchanged.

    python -m goal_gb300.cli primal input.yaml

``primal`` is GoalPrimal (src/main_primal.cpp:68-90): load steps of Newton
(Primal::solve), the functional after each step, States::update, and the
regression check (src/goal_regression.cpp:14-23), with goal's log lines
(`J(uH) = %.15e`, `||R||`, linear iterations). 3D meshes in SCOREC SMB v5 with
their .dmg model and association file (or the package's .npz mesh file);
functionals "avg disp" and "max vm".
"""
from __future__ import annotations

import os
import sys

from . import api, smb, yaml_lite

VALID = {"num steps", "step size", "initial time", "discretization", "dirichlet bcs", "traction bcs",
         "inward bcs", "mechanics", "functional", "primal linear algebra", "adjoint linear algebra",
         "output", "regression", "adjoint mode", "adaptation"}


def _problem(path):
    doc = yaml_lite.load(path)
    if len(doc) != 1:
        raise ValueError("expected one top-level parameter list")
    name, p = next(iter(doc.items()))
    bad = set(p) - VALID
    if bad:
        raise ValueError(f"unknown parameters: {sorted(bad)}")
    return name, p


def _resolve(base, f):
    return f if os.path.isabs(f) else os.path.normpath(os.path.join(base, f))


def primal(path: str, out=print) -> float:
    name, p = _problem(path)
    base = os.path.dirname(os.path.abspath(path))
    dp = p["discretization"]
    mech_p = p["mechanics"]
    mesh_file = _resolve(base, dp["mesh file"])
    if mesh_file.endswith(".npz"):  # the package's own mesh file (goal_gb300.mesh.save_npz)
        from .mesh import load_npz
        mesh = load_npz(mesh_file, list(mech_p["materials"].keys()))
    else:
        mesh = smb.load(_resolve(base, dp["geom file"]), mesh_file, _resolve(base, dp["assoc file"]))
    model = {"neohookean": api.NEOHOOKEAN, "J2": api.J2}.get(mech_p["model"])
    if model is None:
        raise ValueError(f"unknown model: {mech_p['model']}")
    mats = []
    for es in mesh.elem_set_names:
        m = mech_p["materials"][es]
        mats.append([float(m["E"]), float(m["nu"]), float(m.get("K", 0.0)), float(m.get("Y", 0.0)),
                     float(m.get("c0", 0.0))])
    d = api.Disc(mesh)
    mech = api.Mechanics(d, model, mats, stabilization=bool(mech_p.get("stabilization", True)))
    s = api.SolInfo(d)
    dbcs = [(int(v[0]), str(v[1]), str(v[2])) for v in p.get("dirichlet bcs", {}).values()]
    tbcs = [tuple(str(x) for x in v) for v in p.get("traction bcs", {}).values()]
    if p.get("inward bcs"):
        raise ValueError("inward bcs are not supported")
    bcs = api.Bcs(d, dbcs, tbcs)
    fp = p["functional"]
    qoi = {"avg disp": api.QOI_AVG_DISP, "max vm": api.QOI_KS_VM}.get(fp["type"])
    if qoi is None:
        raise ValueError(f"unknown functional type: {fp['type']}")
    rho = float(fp.get("rho", 0.0))
    la = p["primal linear algebra"]
    prm = api.solve_params(krylov_size=min(int(la.get("krylov size", 100)), 200),
                           max_iters=max(int(la.get("max iters", 100)), 2000),
                           tolerance=float(la.get("tolerance", 1e-10)), precision=api.MIXED, inner_iters=30)
    num_steps = int(p["num steps"])
    dt = float(p["step size"])
    t_old = float(p.get("initial time", 0.0))
    t_now = t_old + dt
    J = None
    for step in range(1, num_steps + 1):
        out(f"****** load step: {step}")
        out(f"****** from time: {t_old:f}")
        out(f"****** to time:   {t_now:f}")
        out(f"*** primal solve: {d.num_dofs} dofs")
        r = api.primal_solve(mech, s, bcs, t_now, t_old, int(la["nonlinear max iters"]),
                             float(la["nonlinear tolerance"]), prm)
        for k, nrm in enumerate(r["norms"]):
            out(f" > ({k + 1}) newton iteration")
            out(f" > ||R|| = {nrm:e}")
        J = api.assemble(mech, None, api.NONE, jacobian=False, save_states=False, qoi=qoi, rho=rho)
        out(f" > functional : {fp['type']}")
        out(f" > J(uH) = {J:.15e}")
        mech.update_states()
        t_old, t_now = t_now, t_now + dt
    reg = p.get("regression")
    if reg:
        err = abs(J - float(reg["value"]))
        if not err < float(reg["tolerance"]):
            raise SystemExit(f"regression failed: |{J:.15e} - {float(reg['value']):.15e}| = {err:e}")
        out(f" > regression: |J - value| = {err:e} < {float(reg['tolerance']):e}")
    return J


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    if len(argv) != 2 or argv[0] != "primal":
        print("usage: python -m goal_gb300.cli primal input.yaml", file=sys.stderr)
        return 2
    primal(argv[1])
    return 0


if __name__ == "__main__":
    sys.exit(main())
