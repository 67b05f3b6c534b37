"""CPU oracle of the learned cut-cell fraction model: TEST INFRASTRUCTURE ONLY.

Only tests, the smoke check and the bench's CPU legs import this module, to check the GPU kernels in
sdfibm_gb300/csrc/mlp.cu and classify.cu.  It has no counterpart in the reference, which computes As only with the
apex/pyramid geometry (geometrictools.cpp:47-116).  It restates the model so that the GPU inputs, forward pass,
backward pass and trainer can be compared term by term:

* stencil: the signed distance at the 5 x 5 x 5 lattice of the cell (spacing h/4, vertices included), divided by h;
* P4, P2: the cell cut into 4^3 (2^3) sub-cells, each sub-cell's fraction the exact cube-plane volume under the plane
  fitted to its 8 corner distances (Scardovelli & Zaleski, J. Comput. Phys. 164 (2000)), averaged;
* inputs (16): the stencil values at the 8 vertices (OpenFOAM cellPoints order of a hex, (i,j,k) (i+1,j,k)
  (i,j+1,k) (i+1,j+1,k), then the same at k+1), at the 6 face centres (-x +x -y +y -z +z) and at the centre, then
  logit(clamp(P2)); the prior is logit(clamp(P4)), clamp to [1e-4, 1 - 1e-4];
* network 16 -> 64 -> 64 -> 1 with SiLU hidden activations; the predicted fraction is sigmoid(prior + o) with o the
  network output;
* numerics of the GPU kernels: the two hidden layers are BF16 x BF16 tensor-core products with FP32
  accumulation, W1 and W2 are rounded to BF16, and the inputs and the first hidden activations are carried
  as a hi + lo pair of BF16 values (so they keep ~16 significant bits); biases, the 64 -> 1 output layer and
  the sigmoid are FP32;
* the loss is the mean squared error of the predicted fraction; the backward pass rounds the operands of its
  tensor-core products (dZ2, dZ1, H1, X) to BF16 and sums the bias gradients and the output layer in FP32.

The pure-Python parts are vectorised numpy; sizes used by the tests are a few thousand cells.
"""
import numpy as np

N_IN = 16
N_FEAT = 17     # rows of a feature record: the 16 inputs, then the prior logit
N_H = 64
N_PARAM = N_H * N_IN + N_H + N_H * N_H + N_H + N_H + 1  # 5313

# flat parameter layout, shared with include/sdfibm_mlp.h
OFF_W1 = 0                        # W1[64][16], row = hidden unit
OFF_B1 = OFF_W1 + N_H * N_IN      # b1[64]
OFF_W2 = OFF_B1 + N_H             # W2[64][64], row = output unit
OFF_B2 = OFF_W2 + N_H * N_H       # b2[64]
OFF_W3 = OFF_B2 + N_H             # w3[64]
OFF_B3 = OFF_W3 + N_H             # b3


def unpack(p):
    p = np.asarray(p, dtype=np.float32)
    assert p.shape == (N_PARAM,)
    W1 = p[OFF_W1:OFF_B1].reshape(N_H, N_IN)
    b1 = p[OFF_B1:OFF_W2]
    W2 = p[OFF_W2:OFF_B2].reshape(N_H, N_H)
    b2 = p[OFF_B2:OFF_W3]
    w3 = p[OFF_W3:OFF_B3]
    b3 = p[OFF_B3]
    return W1, b1, W2, b2, w3, b3


def pack(W1, b1, W2, b2, w3, b3):
    return np.concatenate([np.ravel(W1), b1, np.ravel(W2), b2, w3, [b3]]).astype(np.float32)


def init_params(seed=0):
    """He-style initialisation used by the trainer (uniform, fan-in scaled)."""
    rng = np.random.default_rng(seed)
    W1 = rng.uniform(-1, 1, (N_H, N_IN)) * np.sqrt(3.0 / N_IN)
    W2 = rng.uniform(-1, 1, (N_H, N_H)) * np.sqrt(3.0 / N_H)
    w3 = rng.uniform(-1, 1, N_H) * np.sqrt(3.0 / N_H)
    return pack(W1, np.zeros(N_H), W2, np.zeros(N_H), w3, 0.0)


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even); returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def split(x):
    hi = bf16(x)
    lo = bf16(np.asarray(x, np.float32) - hi)
    return hi, lo


def sigmoid(z):
    with np.errstate(over="ignore"):
        return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * sigmoid(z)


def dsilu(z):
    s = sigmoid(z)
    return s * (1.0 + z * (1.0 - s))


PRIOR_CLAMP = 1e-4


def plane_fraction(X):
    """Exact solid fraction under the plane fitted to the vertex distances (FP64, vectorised)."""
    f = np.asarray(X, np.float64)[:, :8]
    n = np.stack([0.25 * (((f[:, 1] - f[:, 0]) + (f[:, 3] - f[:, 2])) + ((f[:, 5] - f[:, 4]) + (f[:, 7] - f[:, 6]))),
                  0.25 * (((f[:, 2] - f[:, 0]) + (f[:, 3] - f[:, 1])) + ((f[:, 6] - f[:, 4]) + (f[:, 7] - f[:, 5]))),
                  0.25 * (((f[:, 4] - f[:, 0]) + (f[:, 5] - f[:, 1])) + ((f[:, 6] - f[:, 2]) + (f[:, 7] - f[:, 3])))],
                 1)
    d = 0.5 * n.sum(1) - f.mean(1)
    d = d - np.minimum(n, 0).sum(1)
    m = np.abs(n)
    s = m.sum(1)
    out = np.where(d > 0, 1.0, 0.0)
    ok = s > 0
    with np.errstate(divide="ignore", invalid="ignore"):
        a = np.where(ok, d / np.where(ok, s, 1.0), 0.0)
        ms = np.sort(m / np.where(ok, s, 1.0)[:, None], 1)
        flip = a > 0.5
        al = np.where(flip, 1 - a, a)
        m1, m2, m3 = ms[:, 0], ms[:, 1], ms[:, 2]
        m12 = m1 + m2
        r1 = al ** 3 / (6 * m1 * m2 * m3)
        r2 = al * (al - m1) / (2 * m2 * m3) + m1 * m1 / (6 * m2 * m3)
        r3 = (al * al * (3 * m12 - al) + m1 * m1 * (m1 - 3 * al) + m2 * m2 * (m2 - 3 * al)) / (6 * m1 * m2 * m3)
        r4 = (al * al * (3 - 2 * al) + m1 * m1 * (m1 - 3 * al) + m2 * m2 * (m2 - 3 * al) +
              m3 * m3 * (m3 - 3 * al)) / (6 * m1 * m2 * m3)
        r5 = (2 * al - m12) / (2 * m3)
        v = np.where(al < m1, r1, np.where(al < m2, r2, np.where(al < np.minimum(m3, m12), r3,
                                                                  np.where(m3 < m12, r4, r5))))
        v = np.clip(v, 0.0, 1.0)
        v = np.where(flip, 1 - v, v)
    v = np.where(a <= 0, 0.0, np.where(a >= 1, 1.0, v))
    return np.where(ok, v, out)


def _idx(i, j, k):
    return i + 5 * (j + 5 * k)


# stencil points of the 15 distance inputs: vertices (cellPoints order), face centres -x +x -y +y -z +z, centre
INPUT_POINTS = ([_idx(4 * (v & 1), 4 * ((v >> 1) & 1), 4 * (v >> 2)) for v in range(8)] +
                [_idx(0, 2, 2), _idx(4, 2, 2), _idx(2, 0, 2), _idx(2, 4, 2), _idx(2, 2, 0), _idx(2, 2, 4)] +
                [_idx(2, 2, 2)])


def subcell_prior(phi125, n):
    """Mean planar fraction of the n^3 sub-cells (n = 1, 2 or 4) of cells given by their 5^3 stencils [m, 125]."""
    G = np.asarray(phi125, np.float64).reshape(-1, 5, 5, 5)   # [cell][k][j][i]
    d = 4 // n
    tot = np.zeros(G.shape[0])
    for c in range(n):
        for b in range(n):
            for a in range(n):
                f = np.stack([G[:, (c + dk) * d, (b + dj) * d, (a + di) * d]
                              for dk in (0, 1) for dj in (0, 1) for di in (0, 1)], 1)
                tot += plane_fraction(f)
    return tot / n ** 3


def _logit_clamped(v):
    v = np.clip(v, PRIOR_CLAMP, 1 - PRIOR_CLAMP)
    return np.log(v / (1 - v))


def features(phi125):
    """Feature records [m, 17] (16 inputs, then the prior) of cells given by their stencils [m, 125] (phi / h)."""
    phi = np.asarray(phi125, np.float64)
    p4, p2 = subcell_prior(phi, 4), subcell_prior(phi, 2)
    return np.concatenate([phi[:, INPUT_POINTS], _logit_clamped(p2)[:, None], _logit_clamped(p4)[:, None]],
                          1).astype(np.float32)


def band_score(X):
    """|P4 - P2| of the clamped reconstructions, from feature records [m, 17]."""
    X = np.asarray(X, np.float64)
    return np.abs(sigmoid(X[:, 16]) - sigmoid(X[:, 15]))


def forward(p, X, return_all=False, exact=False):
    """Predicted fraction of each cell.  X: [n, 17] float32 feature records (inputs, prior).  FP64 accumulation of
    the FP32-exact products.

    exact=True drops every rounding (FP64 throughout): the plain function, used to check the backward algebra."""
    W1, b1, W2, b2, w3, b3 = unpack(p) if not exact else [np.asarray(t, np.float64) for t in unpack_f64(p)]
    if exact:
        z1 = np.asarray(X, np.float64)[:, :N_IN] @ W1.T + b1
        h1 = silu(z1)
        z2 = h1 @ W2.T + b2
        h2 = silu(z2)
        o = h2 @ w3 + b3
        a = sigmoid(np.asarray(X, np.float64)[:, N_IN] + o)
        if return_all:
            return dict(z1=z1, h1=h1, z2=z2, h2=h2, o=o, a=a)
        return a
    W1b = bf16(W1).astype(np.float64)
    W2b = bf16(W2).astype(np.float64)
    xh, xl = split(np.asarray(X, np.float32)[:, :N_IN])
    z1 = (xh.astype(np.float64) + xl.astype(np.float64)) @ W1b.T + b1
    h1 = silu(z1.astype(np.float32)).astype(np.float32)
    hh, hl = split(h1)
    z2 = (hh.astype(np.float64) + hl.astype(np.float64)) @ W2b.T + b2
    z2 = z2.astype(np.float32)
    h2 = silu(z2).astype(np.float32)
    o = h2.astype(np.float64) @ w3.astype(np.float64) + b3
    a = sigmoid(np.asarray(X, np.float32)[:, N_IN].astype(np.float64) + o)
    if return_all:
        return dict(z1=z1.astype(np.float32), h1=h1, z2=z2, h2=h2, o=o, a=a)
    return a


def unpack_f64(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(N_H, N_IN), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(N_H, N_H),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def loss_grad(p, X, y, exact=False):
    """Loss = mean((a - y)^2) and its gradient; returns (loss, grad[N_PARAM]).

    exact=True: the FP64 gradient of the unrounded function (checked against finite differences)."""
    if exact:
        W1, b1, W2, b2, w3, b3 = unpack_f64(p)
        n = X.shape[0]
        r = forward(p, X, return_all=True, exact=True)
        a = r["a"]
        d = a - y
        dz3 = (2.0 / n) * d * a * (1.0 - a)
        dZ2 = dz3[:, None] * w3[None, :] * dsilu(r["z2"])
        dZ1 = (dZ2 @ W2) * dsilu(r["z1"])
        g = np.concatenate([(dZ1.T @ np.asarray(X, np.float64)[:, :N_IN]).ravel(), dZ1.sum(0), (dZ2.T @ r["h1"]).ravel(),
                            dZ2.sum(0), r["h2"].T @ dz3, [dz3.sum()]])
        return float(np.mean(d * d)), g
    W1, b1, W2, b2, w3, b3 = unpack(p)
    n = X.shape[0]
    r = forward(p, X, return_all=True)
    a = r["a"]
    d = a - y
    loss = float(np.mean(d * d))
    dz3 = (2.0 / n) * d * a * (1.0 - a)                                   # [n]
    dw3 = r["h2"].astype(np.float64).T @ dz3
    db3 = dz3.sum()
    dZ2 = (dz3[:, None] * w3[None, :].astype(np.float64) * dsilu(r["z2"].astype(np.float64))).astype(np.float32)
    db2 = dZ2.astype(np.float64).sum(0)
    dZ2b = bf16(dZ2).astype(np.float64)
    dW2 = dZ2b.T @ bf16(r["h1"]).astype(np.float64)
    dH1 = dZ2b @ bf16(W2).astype(np.float64)
    dZ1 = (dH1 * dsilu(r["z1"].astype(np.float64))).astype(np.float32)
    db1 = dZ1.astype(np.float64).sum(0)
    dW1 = bf16(dZ1).astype(np.float64).T @ bf16(np.asarray(X, np.float32)[:, :N_IN]).astype(np.float64)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dw3, [db3]])
    return loss, g


def adam_step(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (t counts from 1), FP32 state as in the device kernel."""
    m = (b1 * m + (1 - b1) * g).astype(np.float32)
    v = (b2 * v + (1 - b2) * g * g).astype(np.float32)
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return (p - lr * mh / (np.sqrt(vh) + eps)).astype(np.float32), m, v
