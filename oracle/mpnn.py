"""CPU restatement of the learned block-Jacobi correction -- TEST INFRASTRUCTURE ONLY.

The network has no counterpart in the reference (goal uses MueLu AMG,
src/goal_linear_solve.cpp:59-65); this module is the independent numpy
statement of the CUDA forward/backward kernels, used to check their outputs
and gradients.

Graph: nodes of the mesh, edges = off-diagonal 4x4 blocks of the matrix.
Everything the network sees is in the dof-scaled space A^ = S A S with
S = diag(|a_ii|^-1/2), where displacement and pressure rows are comparable.
  x_n      = [D^_n (16), log10 max|D_n| - mean, offdiag/diag ratio of A^,
              fraction of Dirichlet rows, (deg-1)/16]                  (20)
  e_nm     = A^_nm                                                     (16)
  h0       = relu(W0 x + b0)                                          (32)
  layer l  : t_nm = We_l [e_nm; h_m] + be_l ; agg_n = mean_m relu(t_nm)
             h_n <- h_n + relu(Wu_l [h_n; agg_n] + bu_l)                (3 layers)
  C_n      = Wd h_n + bd      = W_n, a 4x4 block in the scaled space, with
             the rows and columns of Dirichlet (identity) rows zeroed  (16)
Preconditioner: two block-Jacobi sweeps, the second one weighted per node,
  z = D^-1 r,   P r = z + S W S^-1 D^-1 (r - A z)
i.e. P = D^-1 + B (I - A D^-1) with B_n = S_n W_n S_n^-1 D_n^-1. W = 0 (the
untrained network: the decoder starts at zero) is plain block-Jacobi.
Loss for probes w_i (scaled residual space, Dirichlet rows zeroed): with
v_i = S^-1 w_i for even i and v_i = A D^-1 S^-1 w_i for odd i (weighted toward
the high end of the spectrum, the part a node-local preconditioner acts on),
  L = sum_i |S (v_i - A P v_i)|^2 / |S v_i|^2.
Weights are used rounded to bfloat16 (round to nearest even); all sums in float32.
The edge messages' inputs [e_nm; h_m] enter the product with We as two
bfloat16 terms, x = bf16(x) + bf16(x - bf16(x)) (the CUDA forward multiplies
them on the tensor cores in that form).
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


def split_bf16(a):
    """x as the sum of two bfloat16 terms, hi = bf16(x) + lo = bf16(x - hi),
    in float32 (identity when ROUND_BF16 is off)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    if not ROUND_BF16:
        return a
    hi = bf16(a)
    return (hi + bf16(a - hi)).astype(np.float32)


def features(brow_ptr, bcol, diag, A):
    """A: (nnzb, 4, 4) float64 blocks. Returns x (N,20) f32, e (nnzb,16) f32,
    sd (N,4) f64 = |a_ii|^-1/2, Dinv (N,4,4), dirichlet (N,4) bool."""
    N = len(brow_ptr) - 1
    D = A[diag]
    dd = np.abs(np.einsum("nii->ni", D))
    sd = np.where(dd > 0, 1.0 / np.sqrt(np.where(dd > 0, dd, 1.0)), 1.0)
    rows = np.repeat(np.arange(N), np.diff(brow_ptr))
    off = bcol != rows
    Ah = A * sd[rows][:, :, None] * sd[bcol][:, None, :]
    Dh = Ah[diag]
    s = np.abs(D).reshape(N, 16).max(axis=1)
    s = np.where(s > 0, s, 1.0)
    offn = np.zeros(N)
    np.add.at(offn, rows[off], np.sqrt((Ah[off] ** 2).sum(axis=(1, 2))))
    dn = np.sqrt((Dh ** 2).sum(axis=(1, 2)))
    # Dirichlet row: a unit row of the diagonal block with no off-diagonal entries
    offr = np.zeros((N, 4))
    np.add.at(offr, rows[off], np.abs(A[off]).sum(axis=2))
    unit = np.abs(D - np.eye(4)[None]).max(axis=2) == 0
    dirichlet = unit & (offr == 0)
    ls = np.log10(s)
    x = np.zeros((N, NF))
    x[:, :16] = Dh.reshape(N, 16)
    x[:, 16] = ls - ls.mean()
    x[:, 17] = offn / np.where(dn > 0, dn, 1.0)
    x[:, 18] = dirichlet.sum(axis=1) / 4.0
    x[:, 19] = (np.diff(brow_ptr) - 1) / 16.0
    e = Ah.reshape(-1, 16)
    Dinv = np.linalg.inv(D)
    return x.astype(np.float32), e.astype(np.float32), sd, Dinv, dirichlet


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
        inp = split_bf16(np.concatenate([e[off], h[bcol[off]]], axis=1))
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


def masked(C, dirichlet):
    keep = (~dirichlet).astype(np.float64)
    return C.reshape(-1, 4, 4).astype(np.float64) * keep[:, :, None] * keep[:, None, :]


def blocks(C, sd, Dinv, dirichlet):
    """B_n = S_n W_n S_n^-1 D_n^-1 (the weighted second sweep)."""
    W = masked(C, dirichlet)
    return np.einsum("nik,nkj->nij", sd[:, :, None] * W / sd[:, None, :], Dinv)


def apply_P(brow_ptr, bcol, A, Dinv, B, r):
    z = np.einsum("nij,nj->ni", Dinv, r.reshape(-1, 4)).ravel()
    u = r - apply_bsr(brow_ptr, bcol, A, z)
    return z + np.einsum("nij,nj->ni", B, u.reshape(-1, 4)).ravel()


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
    """Loss sum_w |S(v - A P v)|^2/|S v|^2 (v = A D^-1 S^-1 w) and its gradient
    w.r.t. the (float32) parameters."""
    params = unflatten(np.asarray(flat, np.float32))
    x, e, sd, Dinv, dirichlet = features(brow_ptr, bcol, diag, A)
    C, cache = forward(params, brow_ptr, bcol, diag, x, e, keep=True)
    W = masked(C, dirichlet)
    N = len(brow_ptr) - 1
    keep = (~dirichlet).astype(np.float64)
    L = 0.0
    dW = np.zeros((N, 4, 4))
    bj = lambda y: np.einsum("nij,nj->ni", Dinv, y.reshape(-1, 4)).ravel()
    for i, w in enumerate(probes):
        q = (w.reshape(-1, 4) * keep / sd).ravel()
        v = apply_bsr(brow_ptr, bcol, A, bj(q)) if i % 2 == 1 else q
        z = bj(v)
        c = bj(v - apply_bsr(brow_ptr, bcol, A, z)).reshape(-1, 4) / sd
        y = z + (sd * np.einsum("nij,nj->ni", W, c)).ravel()
        r = (v - apply_bsr(brow_ptr, bcol, A, y)) * sd.ravel()
        nv = np.sum((v * sd.ravel()) ** 2)
        L += (r @ r) / nv
        g = apply_bsr_t(brow_ptr, bcol, A, r * sd.ravel()).reshape(-1, 4) * sd
        dW += (-2.0 / nv) * np.einsum("ni,nj->nij", g, c)
    dC = (dW * keep[:, :, None] * keep[:, None, :]).reshape(N, 16).astype(np.float32)
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
