"""CPU restatement of the photon guide's network and training loss, for tests
only (the oracle; the library trains the network with its own tensor-core
kernels, friendsrender-r-public_gb300/csrc/fr_guide.cu).

Network: 5 inputs -> 64 -> 64 -> 64 (ReLU) -> 40 outputs = 8 lobes x {raw mean
direction (3), raw concentration, weight logit}.  Lobe k: mean m_k / |m_k|,
concentration 0.5 + softplus(raw) (at most 2000), weight softmax(logits)_k; the
density is the mixture of von Mises-Fisher lobes.  Loss of a sample with
emission input x, direction d and importance I: -I log q(d | x).

The flat parameter layout is the library's: W1[64][5], b1[64], W2[64][64],
b2[64], W3[64][64], b3[64], W4[48][64] (rows 40-47 unused), b4[48].

`gradient(params, samples, bf16=True)` rounds to bfloat16 where the GPU kernels
store tensor-core operands (activations of layers 1-3, the weights of layers
2-4, the output and hidden-layer error signals, the layer-1 inputs of the
weight gradient), so the GPU's gradient sums can be compared closely; with
bf16=False it is the exact float64 gradient.
"""
import numpy as np

IN, HID, LOBES, OUT, OUT_PAD = 5, 64, 8, 40, 48
OFF_W1 = 0
OFF_B1 = OFF_W1 + HID * IN
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID * HID
OFF_W4 = OFF_B3 + HID
OFF_B4 = OFF_W4 + OUT_PAD * HID
N_PARAMS = OFF_B4 + OUT_PAD
KAPPA_MIN, KAPPA_MAX = 0.5, 2000.0


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return dict(W1=p[OFF_W1:OFF_B1].reshape(HID, IN), b1=p[OFF_B1:OFF_W2], W2=p[OFF_W2:OFF_B2].reshape(HID, HID),
                b2=p[OFF_B2:OFF_W3], W3=p[OFF_W3:OFF_B3].reshape(HID, HID), b3=p[OFF_B3:OFF_W4],
                W4=p[OFF_W4:OFF_B4].reshape(OUT_PAD, HID)[:OUT], b4=p[OFF_B4:OFF_B4 + OUT])


def softplus(x):
    return np.where(x > 20.0, x, np.log1p(np.exp(np.minimum(x, 20.0))))


def mixture(o):
    """o: (n, 40) -> means (n,8,3), norms (n,8), kappa (n,8), weights (n,8)."""
    o = o.reshape(-1, LOBES, 5)
    m = o[..., :3]
    nrm = np.maximum(np.linalg.norm(m, axis=-1), 1e-6)
    mu = m / nrm[..., None]
    kraw = o[..., 3]
    kappa = np.minimum(KAPPA_MIN + softplus(kraw), KAPPA_MAX)
    a = o[..., 4]
    w = np.exp(a - a.max(axis=1, keepdims=True))
    w /= w.sum(axis=1, keepdims=True)
    return mu, nrm, kraw, kappa, w


def vmf_log_pdf(kappa, cosang):
    return np.log(kappa / (2 * np.pi)) - np.log1p(-np.exp(-2 * kappa)) + kappa * (cosang - 1.0)


def forward(params, x, rnd=None):
    """Outputs (n, 40) and the activations; rnd rounds tensor-core operands."""
    P = unpack(params)
    r = rnd or (lambda v: np.asarray(v, np.float64))
    h1 = r(np.maximum(x @ P['W1'].T + P['b1'], 0.0))
    h2 = r(np.maximum(h1 @ r(P['W2']).T + P['b2'], 0.0))
    h3 = r(np.maximum(h2 @ r(P['W3']).T + P['b3'], 0.0))
    out = h3 @ r(P['W4']).T + P['b4']
    return out, (h1, h2, h3)


def loss(params, samples):
    x, d, I = samples[:, :5].astype(np.float64), samples[:, 5:8].astype(np.float64), samples[:, 8].astype(np.float64)
    out, _ = forward(params, x)
    mu, _, _, kappa, w = mixture(out)
    lf = np.log(w) + vmf_log_pdf(kappa, np.einsum('nkc,nc->nk', mu, d))
    lmax = lf.max(axis=1, keepdims=True)
    logq = lmax[:, 0] + np.log(np.exp(lf - lmax).sum(axis=1))
    return float(-(I * logq).sum())


def output_grad(out, d, I):
    """dL/d(out) for L = sum -I log q; out (n, 40)."""
    mu, nrm, kraw, kappa, w = mixture(out)
    cs = np.einsum('nkc,nc->nk', mu, d)
    lf = np.log(w) + vmf_log_pdf(kappa, cs)
    lf -= lf.max(axis=1, keepdims=True)
    gam = np.exp(lf)
    gam /= gam.sum(axis=1, keepdims=True)
    e2k = np.exp(-2 * kappa)
    dk = 1.0 / kappa - 2 * e2k / (1 - e2k) + (cs - 1.0)
    sig = 1.0 / (1.0 + np.exp(-kraw))
    clamped = KAPPA_MIN + softplus(kraw) > KAPPA_MAX
    g = np.zeros((len(out), LOBES, 5))
    g[..., 3] = np.where(clamped, 0.0, -I[:, None] * gam * dk * sig)
    g[..., 4] = -I[:, None] * (gam - w)
    gm = d[:, None, :] * (kappa * gam * -I[:, None])[..., None]
    proj = (gm - mu * np.einsum('nkc,nkc->nk', mu, gm)[..., None]) / nrm[..., None]
    g[..., :3] = proj
    return g.reshape(-1, OUT)


def gradient(params, samples, bf16_rounding=True):
    """Gradient of sum_j -I_j log q(d_j | x_j) in the flat layout, and sum I."""
    samples = np.asarray(samples)
    x, d, I = samples[:, :5].astype(np.float64), samples[:, 5:8].astype(np.float64), samples[:, 8].astype(np.float64)
    rnd = bf16 if bf16_rounding else None
    r = rnd or (lambda v: np.asarray(v, np.float64))
    P = unpack(params)
    out, (h1, h2, h3) = forward(params, x, rnd)
    do = r(output_grad(out, d, I))
    dz3 = r((do @ r(P['W4'])) * (h3 > 0))
    dz2 = r((dz3 @ r(P['W3'])) * (h2 > 0))
    dz1 = r((dz2 @ r(P['W2'])) * (h1 > 0))
    g = np.zeros(N_PARAMS)
    g[OFF_W4:OFF_W4 + OUT * HID] = (do.T @ h3).ravel()
    g[OFF_B4:OFF_B4 + OUT] = do.sum(0)
    g[OFF_W3:OFF_B3] = (dz3.T @ h2).ravel()
    g[OFF_B3:OFF_W4] = dz3.sum(0)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    g[OFF_W1:OFF_B1] = (dz1.T @ r(x)).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    return g, float(I.sum())
