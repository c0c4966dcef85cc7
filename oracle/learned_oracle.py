"""ORACLE — test infrastructure only.  NumPy restatement of the learned preconditioner's network: features,
forward pass, loss and gradients (hand-derived, checked against finite differences in tests/), and Adam.  Only
tests/ use it, as the checker of the CUDA forward/backward/Adam kernels (navier_stokes_fem_gb300/csrc/nsf_learn.cu).

The network (the project's own design for the reference's preconditioner slot, include/assembly.h:33-35,
1338-1344): an edge-based message-passing network over the graph of the strictly lower factor pattern (rows
coloured, L_ij for neighbours j of a smaller colour).  Work is done on the diagonally scaled system
A^ = D^-1/2 A D^-1/2; the network outputs L^ with M^ = L^ L^T ~ A^, and the factor of A is L = D^1/2 L^.

    node features  [1, deg/8, sum_j a^_ij, sum_j a^_ij^2]          (j over the off-diagonal pattern of row i)
    edge features  [1, a^_cp, a^_cp^2, (colour(c) - colour(p)) / C]   (edge = lower entry (c, p))
    h0 = relu(fn Wn0 + bn0),   e0 = relu(fe We0 + be0)               (width 32)
    3 layers:  e += relu([e, h_c, h_p] W1e + b1e) W2e + b2e
               m_i = mean of e over the edges incident to i
               h += relu([h, m] W1n + b1n) W2n + b2n
    L^_cp = e . wde + bde,   L^_ii = softplus(h . wdn + bdn)
    loss = || L^ L^T x^ - b^ ||^2 / || b^ ||^2,   x^ = D^1/2 x,  b^ = D^-1/2 b

The dense layers run in BF16 with FP32 accumulation on the GPU; `bf16=True` rounds their inputs and weights the
same way here.
"""
import numpy as np
import scipy.sparse as sp

H = 32
LAYERS = 3
FN = 4
FE = 4

SHAPES = [("Wn0", (FN, H)), ("bn0", (H,)), ("We0", (FE, H)), ("be0", (H,))]
for _l in range(LAYERS):
    SHAPES += [(f"W1e{_l}", (3 * H, H)), (f"b1e{_l}", (H,)), (f"W2e{_l}", (H, H)), (f"b2e{_l}", (H,)),
               (f"W1n{_l}", (2 * H, H)), (f"b1n{_l}", (H,)), (f"W2n{_l}", (H, H)), (f"b2n{_l}", (H,))]
SHAPES += [("wde", (H,)), ("bde", (1,)), ("wdn", (H,)), ("bdn", (1,))]
SOFTPLUS_ONE = float(np.log(np.e - 1.0))      # softplus(SOFTPLUS_ONE) = 1


def param_count():
    return int(sum(np.prod(s) for _, s in SHAPES))


def unflatten(theta):
    out, k = {}, 0
    for name, shape in SHAPES:
        size = int(np.prod(shape))
        out[name] = theta[k:k + size].reshape(shape)
        k += size
    return out


def init_params(seed):
    """He-style initial weights; the decoder starts at L^ = I (M = diag(A), the Jacobi preconditioner)."""
    rng = np.random.default_rng(seed)
    theta = []
    for name, shape in SHAPES:
        if name.startswith("W"):
            fan_in = shape[0]
            w = rng.standard_normal(shape) * np.sqrt(2.0 / fan_in)
            if name.startswith("W2"):
                w *= 0.1                                  # residual branches start small
        elif name == "bdn":
            w = np.full(shape, SOFTPLUS_ONE)
        else:
            w = np.zeros(shape)
        theta.append(w.ravel())
    return np.concatenate(theta).astype(np.float32)


class Graph:
    """The lower-pattern graph of one matrix: edges (child c, parent p) in the factor's canonical order."""

    def __init__(self, A, colour, lrp, lci):
        A = A.tocsr()
        n = A.shape[0]
        self.n = n
        self.colours = int(colour.max()) + 1
        rows = np.repeat(np.arange(n), np.diff(lrp))
        self.c = rows.astype(np.int64)
        self.p = np.asarray(lci[: lrp[-1]], np.int64)
        diag = A.diagonal()
        self.sqrt_d = np.sqrt(diag)
        s = 1.0 / self.sqrt_d
        As = A.multiply(s[:, None]).multiply(s[None, :]).tocsr()
        off = As - sp.diags(As.diagonal())
        off = off.tocsr()
        off.eliminate_zeros()
        deg = np.diff(A.indptr) - (diag != 0)          # off-diagonal pattern entries (explicit zeros count)
        self.fn = np.stack([np.ones(n), deg / 8.0, np.asarray(off.sum(axis=1)).ravel(),
                            np.asarray(off.multiply(off).sum(axis=1)).ravel()], axis=1)
        ahat = np.asarray(As[self.c, self.p]).ravel()
        self.fe = np.stack([np.ones(self.c.size), ahat, ahat * ahat,
                            (colour[self.c].astype(float) - colour[self.p]) / self.colours], axis=1)
        self.deg_l = np.bincount(self.c, minlength=n) + np.bincount(self.p, minlength=n)


def _bf(x, on):
    if not on:
        return x
    x = np.asarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16             # round to nearest even, BF16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(theta, g, bf16=False, keep=False):
    """Returns (lower values L^_cp, diagonal L^_ii[, tape])."""
    P = unflatten(np.asarray(theta, np.float64))
    relu = lambda v: np.maximum(v, 0.0)
    t = {}
    h = relu(g.fn @ P["Wn0"] + P["bn0"])
    e = relu(g.fe @ P["We0"] + P["be0"])
    t["h0pre"] = g.fn @ P["Wn0"] + P["bn0"]
    t["e0pre"] = g.fe @ P["We0"] + P["be0"]
    inv = 1.0 / np.maximum(g.deg_l, 1)
    for l in range(LAYERS):
        X = np.concatenate([e, h[g.c], h[g.p]], axis=1)
        pu = _bf(X, bf16) @ _bf(P[f"W1e{l}"], bf16) + P[f"b1e{l}"]
        u = relu(pu)
        e_new = e + _bf(u, bf16) @ _bf(P[f"W2e{l}"], bf16) + P[f"b2e{l}"]
        m = np.zeros((g.n, H))
        np.add.at(m, g.c, e_new)
        np.add.at(m, g.p, e_new)
        m *= inv[:, None]
        Y = np.concatenate([h, m], axis=1)
        pv = _bf(Y, bf16) @ _bf(P[f"W1n{l}"], bf16) + P[f"b1n{l}"]
        v = relu(pv)
        h_new = h + _bf(v, bf16) @ _bf(P[f"W2n{l}"], bf16) + P[f"b2n{l}"]
        t[l] = (e, h, X, pu, u, e_new, m, Y, pv, v)
        e, h = e_new, h_new
    lower = e @ P["wde"] + P["bde"][0]
    tdiag = h @ P["wdn"] + P["bdn"][0]
    diag = np.logaddexp(0.0, tdiag)
    if keep:
        t["eL"], t["hL"], t["tdiag"] = e, h, tdiag
        return lower, diag, t
    return lower, diag


def factor_values(g, lower, diag):
    """The factor of A itself: L = D^1/2 L^ (row scaling)."""
    return g.sqrt_d[g.c] * lower, g.sqrt_d * diag


def loss_and_grad(theta, g, x, b, bf16=False):
    """loss = ||L^ L^T x^ - b^||^2 / ||b^||^2 and its gradient with respect to theta (flat)."""
    P = unflatten(np.asarray(theta, np.float64))
    lower, diag, t = forward(theta, g, bf16, keep=True)
    xh = x * g.sqrt_d
    bh = b / g.sqrt_d
    y = diag * xh
    np.add.at(y, g.p, lower * xh[g.c])
    z = diag * y
    np.add.at(z, g.c, lower * y[g.p])
    rho = z - bh
    bb = bh @ bh
    loss = (rho @ rho) / bb
    gz = 2.0 * rho / bb
    u = diag * gz
    np.add.at(u, g.p, lower * gz[g.c])
    dlower = gz[g.c] * y[g.p] + u[g.p] * xh[g.c]
    ddiag = gz * y + u * xh
    G = {k: np.zeros_like(v) for k, v in P.items()}
    # decoder
    G["wde"] = t["eL"].T @ dlower
    G["bde"] = np.array([dlower.sum()])
    de = np.outer(dlower, P["wde"])
    dt = ddiag / (1.0 + np.exp(-t["tdiag"]))
    G["wdn"] = t["hL"].T @ dt
    G["bdn"] = np.array([dt.sum()])
    dh = np.outer(dt, P["wdn"])
    inv = 1.0 / np.maximum(g.deg_l, 1)
    for l in reversed(range(LAYERS)):
        e, h, X, pu, u_, e_new, m, Y, pv, v = t[l]
        # node update h_new = h + relu(pv) W2n + b2n.  On the GPU the input-gradient products and these layers'
        # weight gradients (with their bias sums) run on the tensor cores with BF16 operands; bf16 reproduces that.
        G[f"W2n{l}"] = _bf(v, bf16).T @ _bf(dh, bf16)
        G[f"b2n{l}"] = _bf(dh, bf16).sum(axis=0)
        dpv = (_bf(dh, bf16) @ _bf(P[f"W2n{l}"], bf16).T) * (pv > 0)
        G[f"W1n{l}"] = _bf(Y, bf16).T @ _bf(dpv, bf16)
        G[f"b1n{l}"] = _bf(dpv, bf16).sum(axis=0)
        dY = _bf(dpv, bf16) @ _bf(P[f"W1n{l}"], bf16).T
        dh_prev = dh + dY[:, :H]
        dm = dY[:, H:] * inv[:, None]
        de_new = de + dm[g.c] + dm[g.p]
        # edge update e_new = e + relu(pu) W2e + b2e
        G[f"W2e{l}"] = _bf(u_, bf16).T @ _bf(de_new, bf16)
        G[f"b2e{l}"] = _bf(de_new, bf16).sum(axis=0)
        dpu = (_bf(de_new, bf16) @ _bf(P[f"W2e{l}"], bf16).T) * (pu > 0)
        G[f"W1e{l}"] = _bf(X, bf16).T @ _bf(dpu, bf16)
        G[f"b1e{l}"] = _bf(dpu, bf16).sum(axis=0)
        dX = _bf(dpu, bf16) @ _bf(P[f"W1e{l}"], bf16).T
        de = de_new + dX[:, :H]
        np.add.at(dh_prev, g.c, dX[:, H:2 * H])
        np.add.at(dh_prev, g.p, dX[:, 2 * H:])
        dh = dh_prev
    dh0 = dh * (t["h0pre"] > 0)
    de0 = de * (t["e0pre"] > 0)
    G["Wn0"] = g.fn.T @ dh0
    G["bn0"] = dh0.sum(axis=0)
    G["We0"] = g.fe.T @ de0
    G["be0"] = de0.sum(axis=0)
    grad = np.concatenate([G[name].ravel() for name, _ in SHAPES])
    return loss, grad


def adam(theta, grad, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (bias-corrected), in place on float32 arrays."""
    m[:] = b1 * m + (1 - b1) * grad
    v[:] = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    theta[:] = theta - lr * mh / (np.sqrt(vh) + eps)
