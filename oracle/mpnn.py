"""CPU restatement of the learned block-Jacobi correction -- TEST INFRASTRUCTURE ONLY.

The network has no counterpart in the reference (goal uses MueLu AMG,
src/goal_linear_solve.cpp:59-65); this module is the independent numpy
statement of the CUDA forward/backward kernels, used to check their outputs
and gradients.

Graph: nodes of the mesh, edges = off-diagonal 4x4 blocks of the matrix.
  s_n      = max |D_n|                      (D_n diagonal block)
  x_n      = [D_n / s_n (16), log10 s_n - mean, offdiag row ratio, dirichlet flag, deg/16]   (20)
  e_nm     = A_nm / sqrt(s_n s_m)           (16)
  h0       = relu(W0 x + b0)                                          (32)
  layer l  : t_nm = We_l [e_nm; h_m] + be_l ; agg_n = mean_m relu(t_nm)
             h_n <- h_n + relu(Wu_l [h_n; agg_n] + bu_l)                (3 layers)
  C_n      = Wd h_n + bd                                              (16)
  P_n      = D_n^-1 + C_n / s_n          (block of the preconditioner, z_n = P_n r_n)
Weights are used rounded to bfloat16 (round to nearest even); all sums in float32.
Loss for probes v:  L = sum_v |v - A P v|^2 / |v|^2.
"""
from __future__ import annotations

import numpy as np

H = 32
NF = 20
NE = 16
NL = 3


def param_shapes():
    shapes = [("W0", (H, NF)), ("b0", (H,))]
    for l in range(NL):
        shapes += [(f"We{l}", (H, NE + H)), (f"be{l}", (H,)), (f"Wu{l}", (H, 2 * H)), (f"bu{l}", (H,))]
    shapes += [("Wd", (16, H)), ("bd", (16,))]
    return shapes


def num_params():
    return sum(int(np.prod(s)) for _, s in param_shapes())


def unflatten(flat):
    out, o = {}, 0
    for name, shp in param_shapes():
        n = int(np.prod(shp))
        out[name] = flat[o:o + n].reshape(shp)
        o += n
    return out


ROUND_BF16 = True


def bf16(a):
    """Round float32 to the nearest bfloat16 (ties to even), returned as float32.
    With ROUND_BF16 False the weights pass through unrounded (finite-difference checks)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    if not ROUND_BF16:
        return a
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def features(brow_ptr, bcol, diag, A):
    """A: (nnzb, 4, 4) float64 blocks. Returns x (N,20) f32, e (nnzb,16) f32, s (N) f64, Dinv (N,4,4)."""
    N = len(brow_ptr) - 1
    D = A[diag]
    s = np.abs(D).reshape(N, 16).max(axis=1)
    s = np.where(s > 0, s, 1.0)
    rows = np.repeat(np.arange(N), np.diff(brow_ptr))
    off = bcol != rows
    offn = np.zeros(N)
    np.add.at(offn, rows[off], np.sqrt((A[off] ** 2).sum(axis=(1, 2))))
    dn = np.sqrt((D ** 2).sum(axis=(1, 2)))
    ls = np.log10(s)
    x = np.zeros((N, NF))
    x[:, :16] = (D / s[:, None, None]).reshape(N, 16)
    x[:, 16] = ls - ls.mean()
    x[:, 17] = offn / np.where(dn > 0, dn, 1.0)
    # Dirichlet row: a row of the node that is a unit vector with no off-diagonal entries
    dir_flag = np.zeros(N)
    for r in range(4):
        unit = (np.abs(D[:, r, :] - np.eye(4)[r]).max(axis=1) == 0)
        offr = np.zeros(N)
        np.add.at(offr, rows[off], np.abs(A[off][:, r, :]).sum(axis=1))
        dir_flag = np.maximum(dir_flag, (unit & (offr == 0)).astype(float))
    x[:, 18] = dir_flag
    x[:, 19] = (np.diff(brow_ptr) - 1) / 16.0
    e = (A / np.sqrt(s[rows] * s[bcol])[:, None, None]).reshape(-1, 16)
    Dinv = np.linalg.inv(D)
    return x.astype(np.float32), e.astype(np.float32), s, Dinv


def forward(params, brow_ptr, bcol, diag, x, e, keep=False):
    p = {k: bf16(v) for k, v in params.items()}
    N = len(brow_ptr) - 1
    rows = np.repeat(np.arange(N), np.diff(brow_ptr))
    off = bcol != rows
    deg = np.maximum(np.bincount(rows[off], minlength=N), 1).astype(np.float32)
    z0 = x @ p["W0"].T + p["b0"]
    h = np.maximum(z0, 0).astype(np.float32)
    cache = {"z0": z0, "h": [h], "t": [], "agg": [], "u": []}
    for l in range(NL):
        inp = np.concatenate([e[off], h[bcol[off]]], axis=1)
        t = inp @ p[f"We{l}"].T + p[f"be{l}"]
        msg = np.maximum(t, 0)
        agg = np.zeros((N, H), np.float32)
        np.add.at(agg, rows[off], msg)
        agg /= deg[:, None]
        u = np.concatenate([h, agg], axis=1) @ p[f"Wu{l}"].T + p[f"bu{l}"]
        h = (h + np.maximum(u, 0)).astype(np.float32)
        cache["t"].append(t)
        cache["agg"].append(agg)
        cache["u"].append(u)
        cache["h"].append(h)
    C = h @ p["Wd"].T + p["bd"]
    if keep:
        cache.update(p=p, rows=rows, off=off, deg=deg)
        return C.astype(np.float32), cache
    return C.astype(np.float32)


def blocks(C, s, Dinv):
    return Dinv + C.reshape(-1, 4, 4).astype(np.float64) / s[:, None, None]


def apply_bsr(brow_ptr, bcol, A, y):
    N = len(brow_ptr) - 1
    rows = np.repeat(np.arange(N), np.diff(brow_ptr))
    out = np.zeros((N, 4))
    np.add.at(out, rows, np.einsum("kij,kj->ki", A, y.reshape(-1, 4)[bcol]))
    return out.ravel()


def apply_bsr_t(brow_ptr, bcol, A, y):
    N = len(brow_ptr) - 1
    rows = np.repeat(np.arange(N), np.diff(brow_ptr))
    out = np.zeros((N, 4))
    np.add.at(out, bcol, np.einsum("kji,kj->ki", A, y.reshape(-1, 4)[rows]))
    return out.ravel()


def loss_and_grad(flat, brow_ptr, bcol, diag, A, probes):
    """Loss sum_v |v - A P v|^2/|v|^2 and its gradient w.r.t. the (float32) parameters."""
    params = unflatten(np.asarray(flat, np.float32))
    x, e, s, Dinv = features(brow_ptr, bcol, diag, A)
    C, cache = forward(params, brow_ptr, bcol, diag, x, e, keep=True)
    P = blocks(C, s, Dinv)
    N = len(brow_ptr) - 1
    L = 0.0
    dP = np.zeros((N, 4, 4))
    for v in probes:
        vn = v.reshape(-1, 4)
        y = np.einsum("nij,nj->ni", P, vn).ravel()
        r = v - apply_bsr(brow_ptr, bcol, A, y)
        w = 1.0 / (v @ v)
        L += w * (r @ r)
        g = -2.0 * w * apply_bsr_t(brow_ptr, bcol, A, r)
        dP += np.einsum("ni,nj->nij", g.reshape(-1, 4), vn)
    dC = (dP / s[:, None, None]).reshape(N, 16).astype(np.float32)
    p = cache["p"]
    rows, off, deg = cache["rows"], cache["off"], cache["deg"]
    grads = {k: np.zeros_like(v, dtype=np.float32) for k, v in params.items()}
    hL = cache["h"][-1]
    grads["Wd"] = dC.T @ hL
    grads["bd"] = dC.sum(axis=0)
    dh = dC @ p["Wd"]
    for l in reversed(range(NL)):
        h = cache["h"][l]
        agg = cache["agg"][l]
        u = cache["u"][l]
        t = cache["t"][l]
        du = dh * (u > 0)
        grads[f"Wu{l}"] = du.T @ np.concatenate([h, agg], axis=1)
        grads[f"bu{l}"] = du.sum(axis=0)
        dcat = du @ p[f"Wu{l}"]
        dh_new = dh + dcat[:, :H]
        dagg = dcat[:, H:]
        dmsg = dagg[rows[off]] / deg[rows[off], None]
        dt = dmsg * (t > 0)
        inp = np.concatenate([cache_e(e, off), h[bcol[off]]], axis=1)
        grads[f"We{l}"] = dt.T @ inp
        grads[f"be{l}"] = dt.sum(axis=0)
        dinp = dt @ p[f"We{l}"]
        np.add.at(dh_new, bcol[off], dinp[:, NE:])
        dh = dh_new
    dz0 = dh * (cache["z0"] > 0)
    grads["W0"] = dz0.T @ x
    grads["b0"] = dz0.sum(axis=0)
    flat_g = np.concatenate([grads[name].ravel() for name, _ in param_shapes()])
    return L, flat_g.astype(np.float64)


def cache_e(e, off):
    return e[off]


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for name, shp in param_shapes():
        if name.startswith("W") and name != "Wd":
            fan_in = shp[1]
            out.append((rng.standard_normal(shp) * np.sqrt(2.0 / fan_in)).astype(np.float32).ravel())
        else:
            out.append(np.zeros(shp, np.float32).ravel())
    return np.concatenate(out)
