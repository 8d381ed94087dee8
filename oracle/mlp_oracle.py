"""CPU oracle of the learned proposal network (test infrastructure only:
tests import it to check the GPU kernels; the product never does).

A numpy restatement of the network of whatprot_gb300/csrc/wp_mlp.cu in
FP64, with BF16 rounding (round to nearest even) applied at the same points
as the GPU: inputs and weights; the hidden activations H1, H2 and the stored
pre-activations Z1, Z2; the logit gradient dL and the pre-activation
gradients dZ2, dZ1.  What remains between the two is the FP32 accumulation
order of the tensor cores."""
import numpy as np
from scipy.special import erf


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_prime(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def forward(params, x):
    """params: dict W1 [H,64], b1, W2 [H,H], b2, W3 [Ppad,H], b3 (FP32
    masters); x [B, TC].  Returns logits [B, Ppad] and the saved tensors."""
    B, TC = x.shape
    X = np.zeros((B, 64))
    X[:, :TC] = x
    X = bf16(X)
    W1, W2, W3 = bf16(params["W1"]), bf16(params["W2"]), bf16(params["W3"])
    Z1 = X @ W1.T + params["b1"]
    H1 = bf16(gelu(Z1))
    Z2 = H1 @ W2.T + params["b2"]
    H2 = bf16(gelu(Z2))
    L = H2 @ W3.T + params["b3"]
    return L, dict(X=X, W1=W1, W2=W2, W3=W3, Z1=bf16(Z1), H1=H1, Z2=bf16(Z2), H2=H2)


def gradients(params, x, labels, P):
    """Mean softmax cross-entropy over the first P classes (rows with label
    < 0 skipped, the mean over all B rows) and its gradients."""
    B = x.shape[0]
    L, s = forward(params, x)
    Lp = L[:, :P]
    mx = Lp.max(axis=1, keepdims=True)
    e = np.exp(Lp - mx)
    p = e / e.sum(axis=1, keepdims=True)
    onehot = np.zeros_like(p)
    ok = labels >= 0
    onehot[np.arange(B)[ok], labels[ok]] = 1.0
    dLp = (p - onehot) / B
    dLp[~ok] = 0.0
    dL = np.zeros_like(L)
    dL[:, :P] = dLp
    dL = bf16(dL)
    loss = np.where(ok, -np.log(np.maximum(p[np.arange(B), np.maximum(labels, 0)], 1e-300)), 0.0)
    g = {}
    g["W3"] = dL.T @ s["H2"]
    g["b3"] = dL.sum(axis=0)
    dH2 = dL @ s["W3"]
    dZ2 = bf16(dH2 * gelu_prime(s["Z2"]))
    g["W2"] = dZ2.T @ s["H1"]
    g["b2"] = dZ2.sum(axis=0)
    dH1 = dZ2 @ s["W2"]
    dZ1 = bf16(dH1 * gelu_prime(s["Z1"]))
    g["W1"] = dZ1.T @ s["X"]
    g["b1"] = dZ1.sum(axis=0)
    return float(loss.mean()), g, L
