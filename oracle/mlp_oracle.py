"""ORACLE -- test infrastructure only.

FP64 numpy restatement of the radial MLP that stands in for the Table pair potential, with its
training loss and the loss's analytic gradient. Tests check the GPU forward, backward and force
kernels against it; nothing in the product imports it. (The surrogate has no counterpart in the
reference; the Table evaluator it replaces is hoomd/md/EvaluatorPairTable.h, restated in
md_oracle.cc.)

Network, per unordered type pair p = (a <= b) and distance r in [r_min, r_cut):

    phi_k(r) = exp(-gamma (r - mu_k)^2),  mu_k = r_min + k h,  h = (r_cut - r_min)/(K - 1),
               gamma = 1 / (2 h^2),  k = 0 .. K-1 (K = 32)
    z1 = W1e E[p] + W1r phi + b1,   h1 = silu(z1)          (64)
    z2 = W2 h1 + b2,                h2 = silu(z2)          (64)
    U  = w3 . h2 + b3
    F  = -dU/dr  (forward-mode: dz1 = W1r dphi, dh1 = silu'(z1) dz1, dz2 = W2 dh1,
                  dh2 = silu'(z2) dz2, dU = w3 . dh2)

Loss over a batch of B samples with targets (U_t, F_t):
    L = (1/B) sum [ (dU + F_t)^2 + lam (U - U_t)^2 ]

Flat parameter layout (float32 on the device; offsets in floats, P = number of type pairs):
    W1e [64 x 16] @ 0, W1r [64 x 32] @ 1024, b1 [64] @ 3072, W2 [64 x 64] @ 3136, b2 [64] @ 7232,
    w3 [64] @ 7296, b3 @ 7360, E [P x 16] @ 7424; total 7424 + 16 P.

Quantisation model of the tensor-core forward (quant="bf16"): E, W1e, W1r, W2, w3 rounded to
bfloat16; phi, dphi, h1, dh1 rounded to bfloat16 where they enter a matrix product; sums in
FP32 or better. quant="bf16x2" keeps those activations as the sum of two bfloat16 numbers.
"""

import numpy as np

EMB, RBF, HID = 16, 32, 64
OFF = dict(W1e=0, W1r=1024, b1=3072, W2=3136, b2=7232, w3=7296, b3=7360, E=7424)


def n_params(n_pairs):
    return OFF["E"] + EMB * n_pairs


def pair_index(a, b, ntypes):
    """Upper-triangle index of the unordered type pair (a, b)."""
    a, b = np.minimum(a, b), np.maximum(a, b)
    return a * ntypes - a * (a - 1) // 2 + (b - a)


def unpack(theta, n_pairs):
    t = np.asarray(theta, np.float64)
    return dict(W1e=t[0:1024].reshape(HID, EMB), W1r=t[1024:3072].reshape(HID, RBF),
                b1=t[3072:3136], W2=t[3136:7232].reshape(HID, HID), b2=t[7232:7296],
                w3=t[7296:7360], b3=t[7360], E=t[7424:7424 + EMB * n_pairs].reshape(n_pairs, EMB))


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    x = np.asarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16x2(x):
    hi = bf16(x)
    return hi + bf16(np.asarray(x, np.float64) - hi)


def init_params(n_pairs, seed=0):
    """Seeded initialisation (uniform fan-in scaling; embedding N(0, 1))."""
    rng = np.random.default_rng(seed)
    t = np.zeros(n_params(n_pairs), np.float32)
    t[0:1024] = rng.uniform(-1, 1, 1024) / np.sqrt(EMB + RBF)
    t[1024:3072] = rng.uniform(-1, 1, 2048) * 2.0 / np.sqrt(EMB + RBF)
    t[3136:7232] = rng.uniform(-1, 1, 4096) * 2.0 / np.sqrt(HID)
    t[7296:7360] = rng.uniform(-1, 1, 64) / np.sqrt(HID)
    t[7424:] = rng.normal(0, 1, EMB * n_pairs)
    return t


def sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu_terms(z):
    s = sigmoid(z)
    f = z * s
    d1 = s * (1.0 + z * (1.0 - s))
    d2 = s * (1.0 - s) * (2.0 + z * (1.0 - 2.0 * s))
    return f, d1, d2


def rbf(r, r_min, r_cut):
    r = np.asarray(r, np.float64)[:, None]
    h = (r_cut - r_min) / (RBF - 1)
    mu = r_min + h * np.arange(RBF)
    g = 1.0 / (2.0 * h * h)
    phi = np.exp(-g * (r - mu) ** 2)
    dphi = -2.0 * g * (r - mu) * phi
    return phi, dphi


def forward(theta, p, r, r_min, r_cut, n_pairs, quant=None):
    """Returns (U, dU/dr, cache) for samples (p, r)."""
    P = unpack(theta, n_pairs)
    q = {None: lambda x: np.asarray(x, np.float64), "bf16": bf16, "bf16x2": bf16x2}[quant]
    wq = (lambda x: np.asarray(x, np.float64)) if quant is None else bf16
    W1e, W1r, W2, w3, E = wq(P["W1e"]), wq(P["W1r"]), wq(P["W2"]), wq(P["w3"]), wq(P["E"])
    phi, dphi = rbf(r, r_min, r_cut)
    phi_q, dphi_q = q(phi), q(dphi)
    e = E[np.asarray(p)]
    z1 = e @ W1e.T + phi_q @ W1r.T + P["b1"]
    dz1 = dphi_q @ W1r.T
    h1, s1, t1 = silu_terms(z1)
    dh1 = s1 * dz1
    h1_q, dh1_q = q(h1), q(dh1)
    z2 = h1_q @ W2.T + P["b2"]
    dz2 = dh1_q @ W2.T
    h2, s2, t2 = silu_terms(z2)
    dh2 = s2 * dz2
    U = h2 @ w3 + P["b3"]
    dU = dh2 @ w3
    cache = dict(e=e, phi=phi_q, dphi=dphi_q, z1=z1, dz1=dz1, h1=h1_q, dh1=dh1_q, s1=s1, t1=t1,
                 z2=z2, dz2=dz2, h2=h2, dh2=dh2, s2=s2, t2=t2, W1e=W1e, W1r=W1r, W2=W2, w3=w3)
    return U, dU, cache


def loss_and_grad(theta, p, r, Ut, Ft, lam, r_min, r_cut, n_pairs, quant=None):
    """Loss and its gradient w.r.t. the flat parameters (straight-through for the rounding)."""
    U, dU, c = forward(theta, p, r, r_min, r_cut, n_pairs, quant)
    B = len(r)
    eU = U - Ut
    eD = dU + Ft
    L = np.mean(eD ** 2 + lam * eU ** 2)
    gU = 2.0 * lam * eU / B
    gD = 2.0 * eD / B
    g = np.zeros(n_params(n_pairs))
    g[7296:7360] = gU @ c["h2"] + gD @ c["dh2"]
    g[7360] = gU.sum()
    g_h2 = gU[:, None] * c["w3"]
    g_dh2 = gD[:, None] * c["w3"]
    g_dz2 = g_dh2 * c["s2"]
    g_z2 = g_h2 * c["s2"] + g_dh2 * c["t2"] * c["dz2"]
    g[3136:7232] = (g_z2.T @ c["h1"] + g_dz2.T @ c["dh1"]).ravel()
    g[7232:7296] = g_z2.sum(0)
    g_h1 = g_z2 @ c["W2"]
    g_dh1 = g_dz2 @ c["W2"]
    g_dz1 = g_dh1 * c["s1"]
    g_z1 = g_h1 * c["s1"] + g_dh1 * c["t1"] * c["dz1"]
    g[0:1024] = (g_z1.T @ c["e"]).ravel()
    g[1024:3072] = (g_z1.T @ c["phi"] + g_dz1.T @ c["dphi"]).ravel()
    g[3072:3136] = g_z1.sum(0)
    gE = g_z1 @ c["W1e"]
    GE = np.zeros((n_pairs, EMB))
    np.add.at(GE, np.asarray(p), gE)
    g[7424:] = GE.ravel()
    return L, g


def pair_forces(theta, pos, types, box_L, ntypes, r_min, r_cut, quant=None):
    """Per-particle forces and energies of the surrogate by brute force over all pairs
    (orthorhombic periodic box; small systems)."""
    pos = np.asarray(pos, np.float64)
    N = len(pos)
    L = np.asarray(box_L, np.float64)
    F = np.zeros((N, 3))
    E = np.zeros(N)
    n_pairs = ntypes * (ntypes + 1) // 2
    for i in range(N - 1):
        d = pos[i] - pos[i + 1:]
        d -= L * np.rint(d / L)
        r = np.sqrt((d * d).sum(1))
        m = (r >= r_min) & (r < r_cut)
        if not m.any():
            continue
        js = np.arange(i + 1, N)[m]
        p = pair_index(np.full(len(js), types[i]), types[js], ntypes)
        U, dU, _ = forward(theta, p, r[m], r_min, r_cut, n_pairs, quant)
        f = (-dU / r[m])[:, None] * d[m]
        F[i] += f.sum(0)
        np.add.at(F, js, -f)
        E[i] += 0.5 * U.sum()
        np.add.at(E, js, 0.5 * U)
    return F, E
