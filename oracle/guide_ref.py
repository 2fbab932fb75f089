"""FP64 restatement of the path-guiding network, for tests only.

Test infrastructure: only tests/ (and bench.py's checks) import it, never the
product path. It restates what renderer_gb300/csrc/guide_net.cuh and guide.cu
compute (the guide has no counterpart in the renderer, which samples BSDFs
only, src/unidipathtracingintegrator.cpp:34-46):

  encoding  position (normalised by the scene box) and (normal + 1) / 2 as
            sin/cos(2^j pi v), j = 0..11, per coordinate; theta / pi and
            phi / 2pi + 1/2 of the outgoing direction as 32 Gaussian bins each
            (sigma = 1 / 32, phi wrapped)
  network   208 -> 64 -> 64 -> 64 -> 40, ReLU, no biases
  output    softmax lobe weights, normalised means, kappa = exp(clamp(b, -4, 9))
  loss      -(1/N) sum w log q(wi), q the vMF mixture

With bf16=True the layer inputs and the weights are rounded to bfloat16 as
the tensor-core kernels do (straight through for the gradient), so the GPU
results can be compared with tight tolerances.
"""
import math

import numpy as np
import torch

K_IN, K_HID, K_OUT, LOBES, BANDS, BLOB = 208, 64, 40, 8, 12, 32
LOGK_MIN, LOGK_MAX = -4.0, 9.0
SHAPES = [(64, 208), (64, 64), (64, 64), (40, 64)]
N_PARAMS = sum(a * b for a, b in SHAPES)


def split(w):
    w = torch.as_tensor(w, dtype=torch.float64)
    out, o = [], 0
    for a, b in SHAPES:
        out.append(w[o:o + a * b].reshape(a, b))
        o += a * b
    return out


def _bf16(x):
    return x + (x.to(torch.bfloat16).to(torch.float64) - x).detach()


def encode(inputs, bounds):
    """inputs (N, 9) point, normal, outgoing direction -> (N, 208) float64."""
    xf = np.asarray(inputs, np.float32)
    x = torch.as_tensor(xf, dtype=torch.float64)
    b = np.asarray(bounds, np.float32)
    ext = b[3:] - b[:3]
    inv = np.where(ext > 0, np.float32(1) / np.where(ext > 0, ext, np.float32(1)), np.float32(0)).astype(np.float32)
    # The normalised coordinates in float32, as the kernels compute them
    # (the highest band multiplies their rounding error by 2^11 pi).
    v = np.clip((xf[:, 0:3] - b[:3]) * inv, 0, 1).astype(np.float32)
    vn = (np.float32(0.5) * (xf[:, 3:6] + np.float32(1))).astype(np.float32)
    vals = torch.as_tensor(np.concatenate([v, vn], 1), dtype=torch.float64)
    feats = []
    for c in range(6):
        for j in range(BANDS):
            a = math.pi * vals[:, c] * (2.0 ** j)
            feats += [torch.sin(a), torch.cos(a)]
    wo = x[:, 6:9]
    theta = torch.acos(torch.clamp(wo[:, 2], -1, 1)) / math.pi
    phi = torch.atan2(wo[:, 1], wo[:, 0]) / (2 * math.pi) + 0.5
    centres = (torch.arange(BLOB, dtype=torch.float64) + 0.5) / BLOB
    dt = (theta[:, None] - centres) * BLOB
    dp = phi[:, None] - centres
    dp = (dp - torch.round(dp)) * BLOB
    return torch.cat([torch.stack(feats, 1), torch.exp(-0.5 * dt * dt), torch.exp(-0.5 * dp * dp)], 1)


def forward(w, x0, bf16=True):
    """Raw outputs (N, 40) of the network on encoded inputs x0."""
    W = split(w)
    r = _bf16 if bf16 else (lambda t: t)
    W = [r(m) for m in W]
    h = r(x0)
    for m in W[:3]:
        h = r(torch.relu(h @ m.T))
    return h @ W[3].T


def decode(o):
    """Raw outputs -> (N, 40) mixture: weights [8], then (mean xyz, kappa) x 8."""
    pi = torch.softmax(o[:, :LOBES], 1)
    m = o[:, 8:32].reshape(-1, LOBES, 3)
    mu = m / torch.linalg.norm(m, dim=2, keepdim=True)
    kap = torch.exp(torch.clamp(o[:, 32:40], LOGK_MIN, LOGK_MAX))
    lobes = torch.cat([mu, kap[:, :, None]], 2).reshape(-1, 4 * LOBES)
    return torch.cat([pi, lobes], 1)


def log_q(o, wi):
    """log of the mixture density of the unit directions wi (N, 3)."""
    logpi = torch.log_softmax(o[:, :LOBES], 1)
    m = o[:, 8:32].reshape(-1, LOBES, 3)
    mu = m / torch.linalg.norm(m, dim=2, keepdim=True)
    kap = torch.exp(torch.clamp(o[:, 32:40], LOGK_MIN, LOGK_MAX))
    c = (mu * wi[:, None, :]).sum(2)
    logf = torch.log(kap) - math.log(2 * math.pi) - torch.log(-torch.expm1(-2 * kap)) + kap * (c - 1)
    return torch.logsumexp(logpi + logf, 1)


def loss_and_grad(w, samples, bounds, bf16=True):
    """Loss -(1/N) sum w log q and its gradient (N_PARAMS,) for samples
    (N, 13): point, normal, outgoing, sampled direction, weight."""
    s = np.asarray(samples, np.float32)
    wt = torch.tensor(np.asarray(w, np.float64), requires_grad=True)
    x0 = encode(s[:, 0:9], bounds)
    o = forward(wt, x0, bf16)
    wi = torch.as_tensor(s[:, 9:12], dtype=torch.float64)
    weight = torch.as_tensor(s[:, 12], dtype=torch.float64)
    loss = -(weight * log_q(o, wi)).sum() / len(s)
    loss.backward()
    return float(loss.detach()), wt.grad.numpy().copy()


def mixture(w, inputs, bounds, bf16=True):
    with torch.no_grad():
        return decode(forward(w, encode(inputs, bounds), bf16)).numpy()


def mixture_pdf(mix, wi):
    """Density of the mixtures (N, 40) at the unit directions wi (N, 3)."""
    mix = np.asarray(mix, np.float64)
    wi = np.asarray(wi, np.float64)
    pi = mix[:, :8]
    lob = mix[:, 8:].reshape(-1, 8, 4)
    c = (lob[:, :, :3] * wi[:, None, :]).sum(2)
    k = lob[:, :, 3]
    f = k / (2 * math.pi * (-np.expm1(-2 * k))) * np.exp(k * (c - 1))
    return (pi * f).sum(1)
