"""Radial MLP surrogate of a multi-type tabulated pair potential (``md.pair.Table``).

One network serves every type pair: a learned 16-wide embedding of the unordered type pair and
32 Gaussian radial features of r feed two hidden layers of 64 SiLU units and a scalar energy;
the force is -dU/dr, differentiated analytically through the same layers. Inference runs on BF16
tensor cores with FP32 accumulation (``md.pair.TableSurrogate``); training runs the project's own
FP32 forward/backward kernels and Adam on the GPU (gb_mlp_loss_grad / gb_mlp_adam in
include/hoomd_gb300.h).

Workflow::

    sur = Surrogate.from_table(table_params, types, r_min, r_cut)   # teacher: the Table
    samples = sur.sample_pairs(snapshots)       # pairs seen in plain-Table NVT trajectories
    sur.fit(samples, steps=20000)
    lj = md.pair.TableSurrogate(nlist=cell, surrogate=sur)
"""

import os

import numpy as np

from hoomd_gb300._native import _hoomd_gb300 as _cpp


def pair_index(a, b, ntypes):
    """Index of the unordered type pair (a, b) in the embedding table."""
    a, b = np.minimum(a, b), np.maximum(a, b)
    return a * ntypes - a * (a - 1) // 2 + (b - a)


class Surrogate:
    """The network, its teacher tables and its training state."""

    def __init__(self, ntypes, r_min, r_cut, seed=0):
        self.ntypes = int(ntypes)
        self.r_min, self.r_cut = float(r_min), float(r_cut)
        self._cpp = _cpp.MlpSurrogate(self.ntypes, self.r_min, self.r_cut, int(seed))
        self.tables = None
        self.history = []

    @property
    def n_pairs(self):
        return self.ntypes * (self.ntypes + 1) // 2

    @classmethod
    def from_table(cls, params, types, r_min, r_cut, seed=0):
        """``params``: {(type_a, type_b): dict(r_min, U, F)} as ``md.pair.Table.params`` takes
        them, every unordered pair present, all with the same r_min and width."""
        types = list(types)
        sur = cls(len(types), r_min, r_cut, seed)
        width = None
        U = F = None
        for (a, b), v in params.items():
            i, j = types.index(a), types.index(b)
            u, f = np.asarray(v["U"], np.float64), np.asarray(v["F"], np.float64)
            if width is None:
                width = len(u)
                U = np.zeros((sur.n_pairs, width))
                F = np.zeros((sur.n_pairs, width))
            if len(u) != width or abs(float(v["r_min"]) - sur.r_min) > 1e-12:
                raise ValueError("every table needs the same r_min and width")
            k = pair_index(i, j, sur.ntypes)
            U[k], F[k] = u, f
        sur.tables = (U, F)
        return sur

    def table_values(self, pair, r):
        """The teacher: Table's linear interpolation (hoomd/md/EvaluatorPairTable.h:151-194,
        V = F = 0 past the last point) at (pair, r), in float64."""
        U, F = self.tables
        width = U.shape[1]
        dr = (self.r_cut - self.r_min) / width
        x = (np.asarray(r, np.float64) - self.r_min) / dr
        i = np.clip(np.floor(x).astype(np.int64), 0, width - 1)
        f = x - i
        nxt = np.minimum(i + 1, width - 1)
        last = i + 1 >= width
        u0, f0 = U[pair, i], F[pair, i]
        u1 = np.where(last, 0.0, U[pair, nxt])
        f1 = np.where(last, 0.0, F[pair, nxt])
        return u0 + f * (u1 - u0), f0 + f * (f1 - f0)

    def sample_pairs(self, frames, anchors=20000, seed=0):
        """Training samples from trajectory frames: ``frames`` is a list of (positions (N, 3),
        typeid (N,), box lengths (3,)) of a cubic or orthorhombic periodic box, or the name of a
        GSD trajectory (every frame, through ``gsd_frames``). For ``anchors``
        random particles per frame, every neighbour within [r_min, r_cut) gives one sample
        (pair index, r, U, F) with the Table's values as targets."""
        from scipy.spatial import cKDTree
        if isinstance(frames, (str, os.PathLike)):
            frames = gsd_frames(frames)
        rng = np.random.default_rng(seed)
        P, R = [], []
        for pos, typeid, L in frames:
            L = np.asarray(L, np.float64)
            x = np.mod(np.asarray(pos, np.float64) + L / 2, L)
            tree = cKDTree(x, boxsize=L)
            idx = rng.choice(len(x), min(anchors, len(x)), replace=False)
            nbrs = tree.query_ball_point(x[idx], self.r_cut)
            for a, js in zip(idx, nbrs):
                js = np.asarray(js, np.int64)
                js = js[js != a]
                d = x[a] - x[js]
                d -= L * np.rint(d / L)
                r = np.sqrt((d * d).sum(1))
                m = r >= self.r_min
                P.append(pair_index(typeid[a], typeid[js[m]], self.ntypes))
                R.append(r[m])
        P = np.concatenate(P).astype(np.uint32)
        R = np.concatenate(R)
        U, F = self.table_values(P, R)
        return dict(pair=P, r=R.astype(np.float32), U=U.astype(np.float32),
                    F=F.astype(np.float32))

    def fit(self, samples, steps=20000, batch=8192, lr=3e-3, lr_min=3e-5, lam=0.1, quant=1,
            report=500):
        """Adam with a cosine schedule on the samples; rounding-aware (quant=1: bfloat16 weights
        and activations in the training forward, straight-through gradients)."""
        self._cpp.setSamples(samples["pair"], samples["r"], samples["U"], samples["F"])
        losses = self._cpp.train(int(steps), int(batch), float(lr), float(lr_min), float(lam),
                                 int(quant), int(report))
        self.history += list(losses)
        return losses

    def evaluate(self, pair, r):
        """(U, F = -dU/dr) from the tensor-core path."""
        U, dU = self._cpp.eval(np.asarray(pair, np.uint32), np.asarray(r, np.float32))
        return U, -dU

    @property
    def params(self):
        return self._cpp.getParams()

    @params.setter
    def params(self, theta):
        self._cpp.setParams(np.asarray(theta, np.float32))

    def save(self, path):
        np.savez(path, theta=self.params, ntypes=self.ntypes, r_min=self.r_min, r_cut=self.r_cut)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        sur = cls(int(d["ntypes"]), float(d["r_min"]), float(d["r_cut"]))
        sur.params = d["theta"]
        return sur


def gsd_frames(filename, start=0, stop=None, step=1):
    """(positions, typeid, box lengths) of frames of a ``hoomd``-schema GSD trajectory (as written
    by hoomd.write.GSD), the input of ``Surrogate.sample_pairs``."""
    from hoomd_gb300.gsd import hoomd as gh
    out = []
    with gh.open(filename, "r") as traj:
        for fr in traj[start:stop:step]:
            box = np.asarray(fr.configuration.box, np.float64)
            if np.any(box[3:] != 0):
                raise ValueError("training frames need an orthorhombic box")
            out.append((np.asarray(fr.particles.position, np.float64),
                        np.asarray(fr.particles.typeid, np.int64), box[:3]))
    return out
