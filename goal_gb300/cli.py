"""Command-line drivers that read goal's input files unchanged.

    python -m goal_gb300.cli primal input.yaml
    python -m goal_gb300.cli nested input.yaml

``primal`` is GoalPrimal (src/main_primal.cpp:68-90): load steps of Newton
(Primal::solve), the functional after each step, the output, States::update,
and the regression check (src/goal_regression.cpp:14-23), with goal's log lines
(`J(uH) = %.15e`, `||R||`, linear iterations).

``nested`` is GoalNested (src/main_nested.cpp:128-151) for adjoint mode
"uniform": per load step and adaptation cycle the primal solve, the
functional and the output; before every cycle but the last, NestedAdjoint::run
on the uniformly refined mesh (`z.R = %.15e`, `|J(u)-J(uh)| < %.15e`), the
isotropic target size field (src/goal_size_field.cpp) for "target elems" x
"target growth"^(cycle-1), and the adaptation of the mesh to that size
(edge-collapse coarsening, then longest-edge bisection) with the solution and
states carried over (goal_gb300.adapt; goal remeshes with SCOREC ma::adapt).

3D meshes in SCOREC SMB v5 with their .dmg model and association file, the
package's .npz mesh file, or a restart directory written with "write native";
functionals "avg disp" and "max vm".
"""
from __future__ import annotations

import os
import sys

from . import api, output, smb, yaml_lite

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


class _Setup:
    """Disc, Mechanics, SolInfo, BCs, functional and output of an input file."""

    def __init__(self, path):
        self.name, p = _problem(path)
        self.p = p
        base = os.path.dirname(os.path.abspath(path))
        dp = p["discretization"]
        mech_p = p["mechanics"]
        mesh_file = _resolve(base, dp["mesh file"])
        self.restart = None
        if output.is_restart(mesh_file):  # a directory written with "write native"
            mesh, U, states = output.load_restart(mesh_file)
            self.restart = (U, states)
        elif mesh_file.endswith(".npz"):  # the package's own mesh file (goal_gb300.mesh.save_npz)
            from .mesh import load_npz
            mesh = load_npz(mesh_file, list(mech_p["materials"].keys()))
        else:
            mesh = smb.load(_resolve(base, dp["geom file"]), mesh_file, _resolve(base, dp["assoc file"]))
        self.model = {"neohookean": api.NEOHOOKEAN, "J2": api.J2}.get(mech_p["model"])
        if self.model is None:
            raise ValueError(f"unknown model: {mech_p['model']}")
        self.dbcs = [(int(v[0]), str(v[1]), str(v[2])) for v in p.get("dirichlet bcs", {}).values()]
        self.tbcs = [tuple(str(x) for x in v) for v in p.get("traction bcs", {}).values()]
        if p.get("inward bcs"):
            raise ValueError("inward bcs are not supported")
        self.build(mesh)
        if self.restart:
            output.apply_restart(self.mech, *self.restart)
        fp = p["functional"]
        self.qoi_name = fp["type"]
        self.qoi = {"avg disp": api.QOI_AVG_DISP, "max vm": api.QOI_KS_VM}.get(fp["type"])
        if self.qoi is None:
            raise ValueError(f"unknown functional type: {fp['type']}")
        self.rho = float(fp.get("rho", 0.0))
        self.prm = self._linear(p["primal linear algebra"])
        la = p["primal linear algebra"]
        self.newton_iters = int(la["nonlinear max iters"])
        self.newton_tol = float(la["nonlinear tolerance"])
        self.output = output.Output(p.get("output", {}), mesh, self.mech, os.getcwd())

    def build(self, mesh):
        """Disc::build_data, Mechanics, SolInfo and BCs on ``mesh``."""
        mech_p = self.p["mechanics"]
        mats = []
        for es in mesh.elem_set_names:
            m = mech_p["materials"][es]
            mats.append([float(m["E"]), float(m["nu"]), float(m.get("K", 0.0)), float(m.get("Y", 0.0)),
                         float(m.get("c0", 0.0))])
        self.mesh = mesh
        self.d = api.Disc(mesh)
        self.mech = api.Mechanics(self.d, self.model, mats, stabilization=bool(mech_p.get("stabilization", True)))
        self.s = api.SolInfo(self.d)
        self.bcs = api.Bcs(self.d, self.dbcs, self.tbcs)
        if hasattr(self, "output"):
            self.output.mesh, self.output.mech = mesh, self.mech

    def adapt_to(self, size, ratio=1.5):
        """Adapts the mesh to the target size field (coarsening, then
        refinement) and moves the solution and the states onto it (the
        remeshing of Solver::adapt, src/main_nested.cpp:106-126, with goal's
        field transfer)."""
        from . import adapt
        U = self.mech.get_solution().reshape(-1, 4)
        states = {n: self.mech.get_state(w) for n, w, _ in output.STATE_FIELDS
                  if self.model == api.J2 or w == api.SIGMA}
        mesh, tr = adapt.adapt_to_size(self.mesh, size, refine_ratio=ratio)
        U2 = tr.nodal(U)
        st2 = tr.states(states)
        self.build(mesh)
        self.mech.set_solution(U2.ravel())
        ids = {n: w for n, w, _ in output.STATE_FIELDS}
        for k, v in st2.items():
            self.mech.set_state(ids[k], v)

    @staticmethod
    def _linear(la):
        return api.solve_params(krylov_size=min(int(la.get("krylov size", 100)), 200),
                                max_iters=max(int(la.get("max iters", 100)), 2000),
                                tolerance=float(la.get("tolerance", 1e-10)), precision=api.MIXED, inner_iters=30)

    def steps(self):
        num_steps = int(self.p["num steps"])
        dt = float(self.p["step size"])
        t_old = float(self.p.get("initial time", 0.0))
        for step in range(1, num_steps + 1):
            yield step, t_old + dt, t_old
            t_old += dt

    def primal_step(self, step, t_now, t_old, out):
        out(f"****** load step: {step}")
        out(f"****** from time: {t_old:f}")
        out(f"****** to time:   {t_now:f}")
        out(f"*** primal solve: {self.d.num_dofs} dofs")
        out(f"*** at time: {t_now:f}")
        r = api.primal_solve(self.mech, self.s, self.bcs, t_now, t_old, self.newton_iters, self.newton_tol, self.prm)
        for k, nrm in enumerate(r["norms"]):
            out(f" > ({k + 1}) newton iteration")
            out(f" > ||R|| = {nrm:e}")
        J = api.assemble(self.mech, None, api.NONE, jacobian=False, save_states=False, qoi=self.qoi, rho=self.rho)
        out(f" > functional : {self.qoi_name}")
        out(f" > J(uH) = {J:.15e}")
        return J

    def regression(self, J, out):
        reg = self.p.get("regression")
        if reg:
            err = abs(J - float(reg["value"]))
            if not err < float(reg["tolerance"]):
                raise SystemExit(f"regression failed: |{J:.15e} - {float(reg['value']):.15e}| = {err:e}")
            out(f" > regression: |J - value| = {err:e} < {float(reg['tolerance']):e}")


def primal(path: str, out=print) -> float:
    S = _Setup(path)
    J = None
    for step, t_now, t_old in S.steps():
        J = S.primal_step(step, t_now, t_old, out)
        S.output.write(t_now, 0)
        S.mech.update_states()
    S.regression(J, out)
    return J


def nested(path: str, out=print) -> dict:
    S = _Setup(path)
    mode = S.p.get("adjoint mode", "uniform")
    if mode != "uniform":
        raise ValueError(f"adjoint mode {mode!r} is not supported (uniform only)")
    ad = S.p.get("adaptation", {})
    target0 = int(ad.get("target elems", S.mesh.num_elems))
    growth = float(ad.get("target growth", 1.0))
    cycles = int(ad.get("adapt cycles", 1))
    aprm = S._linear(S.p.get("adjoint linear algebra", S.p["primal linear algebra"]))
    J = None
    last = {"cycles": []}
    for step, t_now, t_old in S.steps():
        for cycle in range(cycles + 1):
            J = S.primal_step(step, t_now, t_old, out)
            S.output.write(t_now, cycle)
            rec = {"step": step, "cycle": cycle, "elements": S.mesh.num_elems, "J": J}
            if cycle < cycles:
                na = api.NestedAdjoint(S.mech, S.dbcs, S.tbcs)
                out(f"*** adjoint error estimation: {na.disc.num_dofs} dofs")
                out(f"*** at time: {t_now:f}")
                r = na.run(S.qoi, S.rho, t_now, t_old, aprm)
                out(f" > z.R = {r['eta']:.15e}")
                out(f" > |J(u)-J(uh)| < {r['bound']:.15e}")
                na.close()
                out("*** adaptation")
                out(f"*** at step: ({step})")
                out(f"*** at cycle: ({cycle})")
                target = int(target0 * growth ** (cycle - 1.0))
                size = api.size_field(S.d, r["base_error"], max(1, target))
                S.adapt_to(size)
                out(f" > refined to {S.mesh.num_elems} elements (target {target})")
                rec.update(eta=r["eta"], bound=r["bound"], refined_elements=S.mesh.num_elems)
            last["cycles"].append(rec)
        S.mech.update_states()
    S.regression(J, out)
    last["J"] = J
    return last


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    if len(argv) != 2 or argv[0] not in ("primal", "nested"):
        print("usage: python -m goal_gb300.cli {primal|nested} input.yaml", file=sys.stderr)
        return 2
    {"primal": primal, "nested": nested}[argv[0]](argv[1])
    return 0


if __name__ == "__main__":
    sys.exit(main())
