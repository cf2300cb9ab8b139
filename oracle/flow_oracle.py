"""CPU oracle of the affine-coupling flow used as a learned proposal.

TEST INFRASTRUCTURE ONLY (checker of the device flow kernels in
mcintegratorplusplus_gb300/csrc/mcig_flow.cu).  The reference has no learned proposal;
this module defines the flow the device implements and restates it in numpy.

Flow (RealNVP affine couplings, Dinh et al. 2017):
  D coordinates, d = D/2, L layers, hidden width H.  Layer l takes y, gathers
  a = y[perm_l[:d]] and b = y[perm_l[d:]], runs the MLP
      h1 = relu(a W1 + b1), h2 = relu(h1 W2 + b2), o = h2 W3 + b3,
  s = S tanh(o[:d] / S), t = o[d:], and returns y with
      b <- b exp(s) + t            (generative direction z -> x)
      b <- (b - t) exp(-s)         (density direction x -> z).
  After the layers the base affine x = mu + exp(logsig) y.
  log q(x) = log N(z; 0, I) - sum_l sum(s_l) - sum(logsig).
The MLP GEMMs take bfloat16 inputs (activations and weights) with float
accumulation on the device; `bf16=True` rounds the same values here.

Parameters are one flat float32 vector, per layer W1[d][H], b1[H], W2[H][H],
b2[H], W3[H][2d], b3[2d] (row-major, input index first), then mu[D], logsig[D].
"""
import numpy as np

S_MAX = 3.0


def bf16_round(a):
    """Round float values to bfloat16 (round to nearest even) and back."""
    a32 = np.asarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def permutations(D, L, seed):
    """Coordinate permutation of each layer (same generator as the device code: splitmix64 Fisher-Yates)."""
    mask = (1 << 64) - 1
    perms = []
    for l in range(L):
        s = (seed * 0x9E3779B97F4A7C15 + l + 1) & mask
        p = list(range(D))
        for i in range(D - 1, 0, -1):
            s = (s + 0x9E3779B97F4A7C15) & mask
            z = s
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
            z = z ^ (z >> 31)
            j = z % (i + 1)
            p[i], p[j] = p[j], p[i]
        perms.append(np.array(p, dtype=np.int64))
    return perms


def layout(D, L, H):
    d = D // 2
    sizes = []
    for _ in range(L):
        sizes += [("W1", (d, H)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, 2 * d)), ("b3", (2 * d,))]
    sizes += [("mu", (D,)), ("logsig", (D,))]
    return sizes


def unpack(theta, D, L, H):
    out, layers, off = {}, [], 0
    cur = {}
    for name, shp in layout(D, L, H):
        n = int(np.prod(shp))
        v = np.asarray(theta[off:off + n], dtype=np.float64).reshape(shp)
        off += n
        if name in ("mu", "logsig"):
            out[name] = v
        else:
            cur[name] = v
            if name == "b3":
                layers.append(cur)
                cur = {}
    out["layers"] = layers
    return out


def nparams(D, L, H):
    return sum(int(np.prod(s)) for _, s in layout(D, L, H))


def _mlp(a, w, bf16):
    r = bf16_round if bf16 else (lambda v: v)
    h1 = np.maximum(r(a) @ r(w["W1"]) + w["b1"], 0.0)
    h2 = np.maximum(r(h1) @ r(w["W2"]) + w["b2"], 0.0)
    o = r(h2) @ r(w["W3"]) + w["b3"]
    return h1, h2, o


def forward(theta, z, D, L, H, perms, bf16=True):
    """Generative direction: x = f(z) and log q(x)."""
    P = unpack(theta, D, L, H)
    d = D // 2
    y = np.array(z, dtype=np.float64)
    logdet = np.zeros(y.shape[0])
    for l in range(L):
        pa, pb = perms[l][:d], perms[l][d:]
        a = y[:, pa]
        _, _, o = _mlp(a, P["layers"][l], bf16)
        s = S_MAX * np.tanh(o[:, :d] / S_MAX)
        t = o[:, d:]
        y[:, pb] = y[:, pb] * np.exp(s) + t
        logdet += s.sum(1)
    x = P["mu"] + np.exp(P["logsig"]) * y
    logq = -0.5 * (z * z).sum(1) - 0.5 * D * np.log(2 * np.pi) - logdet - P["logsig"].sum()
    return x, logq


def inverse(theta, x, D, L, H, perms, bf16=True, keep=False):
    """Density direction: z = f^-1(x) and log q(x); keep=True also returns the tape for gradients."""
    P = unpack(theta, D, L, H)
    d = D // 2
    y = (np.asarray(x, dtype=np.float64) - P["mu"]) * np.exp(-P["logsig"])
    logdet = np.zeros(y.shape[0])
    tape = []
    for l in range(L - 1, -1, -1):
        pa, pb = perms[l][:d], perms[l][d:]
        a = y[:, pa]
        h1, h2, o = _mlp(a, P["layers"][l], bf16)
        s = S_MAX * np.tanh(o[:, :d] / S_MAX)
        t = o[:, d:]
        bprime = y[:, pb].copy()
        b = (bprime - t) * np.exp(-s)
        tape.append((l, a, h1, h2, s, t, b))
        y[:, pb] = b
        logdet += s.sum(1)
    z = y
    logq = -0.5 * (z * z).sum(1) - 0.5 * D * np.log(2 * np.pi) - logdet - P["logsig"].sum()
    if keep:
        return z, logq, tape
    return z, logq


def loss_and_grad(theta, x, D, L, H, perms, bf16=True):
    """Loss -mean log q(x) and its gradient with respect to theta (float64), backpropagated
    through the density direction in the order the device kernel uses (bf16 rounding of
    every GEMM input when bf16=True)."""
    r = bf16_round if bf16 else (lambda v: v)
    P = unpack(theta, D, L, H)
    d = D // 2
    B = x.shape[0]
    z, logq, tape = inverse(theta, x, D, L, H, perms, bf16, keep=True)
    loss = -logq.mean()
    grads = {}
    g = z / B  # d loss / d z of 0.5|z|^2 averaged over the batch
    for (l, a, h1, h2, s, t, b) in reversed(tape):  # layers 0 .. L-1
        w = P["layers"][l]
        pa, pb = perms[l][:d], perms[l][d:]
        gb = g[:, pb]
        ga = g[:, pa].copy()
        e = np.exp(-s)
        g_bprime = gb * e
        g_t = -gb * e
        g_s = -gb * b + 1.0 / B
        g_sraw = g_s * (1.0 - (s / S_MAX) ** 2)
        g_o = np.concatenate([g_sraw, g_t], axis=1)
        g_h2 = (r(g_o) @ r(w["W3"]).T) * (h2 > 0)
        gW3 = r(h2).T @ r(g_o)
        gb3 = g_o.sum(0)
        g_h1 = (r(g_h2) @ r(w["W2"]).T) * (h1 > 0)
        gW2 = r(h1).T @ r(g_h2)
        gb2 = g_h2.sum(0)
        g_a = r(g_h1) @ r(w["W1"]).T
        gW1 = r(a).T @ r(g_h1)
        gb1 = g_h1.sum(0)
        grads[l] = dict(W1=gW1, b1=gb1, W2=gW2, b2=gb2, W3=gW3, b3=gb3)
        gnew = np.empty_like(g)
        gnew[:, pa] = ga + g_a
        gnew[:, pb] = g_bprime
        g = gnew
    # base affine: y_L = (x - mu) exp(-logsig)
    yL = (x - P["mu"]) * np.exp(-P["logsig"])
    g_mu = -(g * np.exp(-P["logsig"])).sum(0)
    g_logsig = -(g * yL).sum(0) + 1.0
    flat = []
    for l in range(L):
        for name in ("W1", "b1", "W2", "b2", "W3", "b3"):
            flat.append(grads[l][name].ravel())
    flat += [g_mu, g_logsig]
    return loss, np.concatenate(flat)


def init_params(D, L, H, seed):
    """He-normal hidden weights, zero output layer (the flow starts as the identity)."""
    rng = np.random.default_rng(seed)
    d = D // 2
    parts = []
    for _ in range(L):
        parts += [rng.standard_normal((d, H)) * np.sqrt(2.0 / d), np.zeros(H),
                  rng.standard_normal((H, H)) * np.sqrt(2.0 / H), np.zeros(H),
                  np.zeros((H, 2 * d)), np.zeros(2 * d)]
    parts += [np.zeros(D), np.zeros(D)]
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)
