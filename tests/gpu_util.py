"""Helpers for the GPU parity tests: device buffers from torch, calls through the C ABI
(hoomd_gb300.abi), and conversion of the results for comparison with the oracle."""

import ctypes
import math

import numpy as np
import torch

from hoomd_gb300 import abi
from oracle import oracle as O

c_void = ctypes.c_void_p


def dev(a, dtype=None):
    a = np.ascontiguousarray(a if dtype is None else np.asarray(a, dtype))
    return torch.from_numpy(a.copy()).cuda()


def zeros(n, dtype=torch.int32):
    return torch.zeros(int(n), dtype=dtype, device="cuda")


def p(t):
    return c_void(t.data_ptr()) if t is not None else None


def stream():
    return c_void(torch.cuda.current_stream().cuda_stream)


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def r_matrices(r_cut, r_buff):
    """(r_cut, r_list^2, r_cut max per type) at FP32, as updateRList computes them."""
    rc = np.atleast_2d(np.asarray(r_cut, np.float32))
    rl = np.where(rc > 0, rc + np.float32(r_buff), np.float32(0)).astype(np.float32)
    return rc, (rl * rl).astype(np.float32), rc.max(axis=1).astype(np.float32)


class GpuNlist:
    """Cell list + neighbour list through the C ABI, with the reference's overflow retries."""

    def __init__(self, pos4, box6, r_cut, r_buff, layout="col", deterministic=False, ndim=3):
        """layout: "col", "col4" (column-major, interleaved by 4), "flat" (head list); a trailing
        "w" ("colw", "col4w") withholds the list capacity, which selects the warp-per-cell form
        of the tiled build, and a trailing "_lane" ("col_lane", "col4_lane") asks for the
        lane-per-particle form (one thread per own particle) instead of the default candidate
        stream."""
        L = abi.load()
        self.tpp = 1 if layout.endswith("_lane") else 0
        layout = layout[:-5] if self.tpp else layout
        self.warp_build = layout.endswith("w")
        layout = layout[:-1] if self.warp_build else layout
        self.N = N = len(pos4)
        self.box = abi.make_box(box6[:3], box6[3:6])
        self.pos = dev(np.asarray(pos4, np.float32))
        rc, rlsq, rcmax = r_matrices(r_cut, r_buff)
        self.ntypes = nt = rc.shape[0]
        self.d_rc, self.d_rl, self.d_rcmax = dev(rc.ravel()), dev(rlsq.ravel()), dev(rcmax)
        width = float(np.float32(rc.max()) + np.float32(r_buff))
        self.dim = abi.cell_dims(self.box, ndim, width)
        ncell = int(np.prod(self.dim))
        self.adj = zeros(27 * ncell)
        w = ctypes.c_uint32()
        dims = (ctypes.c_uint32 * 3)(*self.dim)
        abi.check(L.gb_cell_adj_build(dims, ndim, p(self.adj), ctypes.byref(w), stream()), "adj")
        self.adj_w = w.value
        types = O.pos_index_bits(np.asarray(pos4, np.float32)[:, 3], 32)
        self.types = types
        Nmax_cell = max(1, math.ceil(N / ncell))
        while True:
            self.cell_size = zeros(ncell)
            self.xyzf = zeros(4 * ncell * Nmax_cell, torch.float32)
            self.cell_type = zeros(ncell * Nmax_cell) if nt > 1 else None
            self.ccond = zeros(3)
            a = abi.CellListArgs(d_pos=p(self.pos), N=N, box=self.box,
                                 dim=(ctypes.c_uint32 * 3)(*self.dim), Nmax=Nmax_cell,
                                 d_cell_size=p(self.cell_size), d_xyzf=p(self.xyzf),
                                 d_cell_type=p(self.cell_type), d_conditions=p(self.ccond),
                                 deterministic=int(deterministic))
            abi.check(L.gb_cell_list_build(ctypes.byref(a), stream()), "cell list")
            cc = host(self.ccond)
            assert cc[1] == 0 and cc[2] == 0, cc
            if cc[0] > Nmax_cell:
                Nmax_cell = int(cc[0])
                continue
            break
        self.Nmax_cell = Nmax_cell
        Nmax = np.full(nt, 4, np.uint32)
        while True:
            self.d_Nmax = dev(Nmax)
            self.n_neigh = zeros(N)
            self.last_pos = zeros(4 * N, torch.float32)
            self.ncond = zeros(nt)
            self.interleave = 4 if layout == "col4" else 1
            if layout in ("col", "col4"):
                self.stride = (N + 31) // 32 * 32
                self.head = None
                self.nlist = zeros(self.stride * int((Nmax.max() + 3) // 4 * 4))
            else:
                self.stride = 1
                nb = (N + 1023) // 1024
                self.head = zeros(N, torch.int64)
                total = zeros(1 + nb, torch.int64)
                abi.check(L.gb_nlist_head_list(p(self.head), p(total), p(self.pos), N,
                                               p(self.d_Nmax), nt, stream()), "head")
                self.nlist = zeros(max(1, int(host(total)[0])))
            a = abi.NlistArgs(d_nlist=p(self.nlist), d_n_neigh=p(self.n_neigh),
                              d_last_pos=p(self.last_pos), d_conditions=p(self.ncond),
                              d_head_list=p(self.head), stride=self.stride,
                              interleave=self.interleave, d_Nmax=p(self.d_Nmax),
                              d_pos=p(self.pos), N=N, d_cell_size=p(self.cell_size),
                              d_xyzf=p(self.xyzf), d_cell_type=p(self.cell_type),
                              d_cell_adj=p(self.adj), dim=(ctypes.c_uint32 * 3)(*self.dim),
                              Nmax_cell=self.Nmax_cell, adj_width=self.adj_w, box=self.box,
                              d_r_cut=p(self.d_rc), d_r_listsq=p(self.d_rl), ntypes=nt,
                              nlist_capacity=0 if self.warp_build else self.nlist.numel(),
                              threads_per_particle=self.tpp)
            abi.check(L.gb_nlist_build_binned(ctypes.byref(a), stream()), "nlist")
            cond = host(self.ncond)
            over = cond > Nmax
            if not over.any():
                break
            Nmax = np.where(over, np.where(cond > 4, (cond + 3) & ~np.uint32(3), 4),
                            Nmax).astype(np.uint32)
        self.Nmax = Nmax

    def word_index(self):
        """index(i, k) -> word offset of particle i's k-th neighbour in this list's layout."""
        if self.head is None and self.interleave == 4:
            st = self.stride
            return lambda i, k: ((k >> 2) * st + i) * 4 + (k & 3)
        if self.head is None:
            st = self.stride
            return lambda i, k: i + k * st
        hd = host(self.head).astype(np.int64)
        return lambda i, k: hd[i] + k

    def sets(self):
        nn = host(self.n_neigh).astype(np.int64)
        nl = host(self.nlist).astype(np.int64)
        if self.head is None and self.interleave == 4:
            out = []
            for i in range(self.N):
                k = np.arange(nn[i])
                out.append(np.sort(nl[((k >> 2) * self.stride + i) * 4 + (k & 3)]))
            return out
        if self.head is None:
            return [np.sort(nl[i + np.arange(nn[i]) * self.stride]) for i in range(self.N)]
        hd = host(self.head)
        return [np.sort(nl[hd[i]: hd[i] + nn[i]]) for i in range(self.N)]

    def pair_args(self, force, virial, rcutsq, ronsq=None, shift=0, tpp=0):
        a = abi.PairArgs(d_force=p(force), d_virial=p(virial),
                         virial_pitch=self.N if virial is not None else 0, N=self.N,
                         d_pos=p(self.pos), box=self.box, d_n_neigh=p(self.n_neigh),
                         d_nlist=p(self.nlist), d_head_list=p(self.head), stride=self.stride,
                         interleave=self.interleave,
                         d_rcutsq=p(rcutsq), d_ronsq=p(ronsq), ntypes=self.ntypes,
                         shift_mode=shift, compute_virial=int(virial is not None),
                         threads_per_particle=tpp)
        return a


RTOL = 1e-5  # relative tolerance of FP32 forces, energies, virials vs the FP64 oracle


def assert_close_f64(got, ref, rtol=RTOL, what=""):
    """|got - ref| <= rtol |ref| + rtol max|ref| elementwise (a relative bar with an absolute
    floor scaled to the largest reference value)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    floor = rtol * max(np.abs(ref).max(), 1e-30)
    err = np.abs(got - ref)
    bad = err > rtol * np.abs(ref) + floor
    assert not bad.any(), (f"{what}: {bad.sum()} of {bad.size} outside tolerance; worst "
                           f"{err.max():.3e} (ref scale {np.abs(ref).max():.3e})")


def assert_close_cond(got, ref, absref, band=0.0, rtol=RTOL, what=""):
    """|got - ref| <= rtol * absref elementwise, absref being the sum of the magnitudes of the
    terms that make up each value (oracle pair_forces with abs_terms=True), plus a floor of
    1e-7 x its largest value. A sum of n FP32 terms is within about n x 6e-8 x absref of the
    exact sum whatever the order, so this bar is met by any correct FP32 summation of up to
    ~150 terms, where a bar relative to the value itself is not when the terms cancel (dense
    liquids: repulsive pair forces tens of times the net force). ``band`` (oracle pair_forces
    with abs_terms=2) adds the magnitude of the terms of pairs within 1e-6 relative of r_cut^2,
    which two correct FP32 evaluations may count or not where the potential does not vanish at
    r_cut."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    absref = np.asarray(absref, np.float64)
    err = np.abs(got - ref)
    bound = rtol * absref + np.asarray(band, np.float64) + 1e-7 * max(absref.max(), 1e-30)
    bad = err > bound
    assert not bad.any(), (f"{what}: {bad.sum()} of {bad.size} outside rtol x sum|terms|; worst "
                           f"ratio {(err / bound).max():.3f}")


PAD = np.uint32(0xFFFFFFFF)


def padded_sorted_rows(n_neigh, nlist, index, lo, hi):
    """Rows lo..hi-1 of a neighbour list as a (hi-lo, max n) array of sorted indices padded with
    0xFFFFFFFF. ``index(i, k)`` maps particle and slot arrays to word offsets in ``nlist``."""
    nn = np.asarray(n_neigh[lo:hi], np.int64)
    K = int(nn.max()) if len(nn) else 0
    i = np.arange(lo, hi, dtype=np.int64)[:, None]
    k = np.arange(K, dtype=np.int64)[None, :]
    valid = k < nn[:, None]
    idx = np.where(valid, index(i, k), 0)
    rows = np.where(valid, nlist[idx], PAD).astype(np.uint32)
    rows.sort(axis=1)
    return rows


def compare_neighbor_sets(nn_a, nl_a, index_a, nn_b, nl_b, index_b, chunk=65536):
    """Indices of the particles whose neighbour sets differ between two lists (vectorised over
    chunks of particles, so a million-particle list compares in seconds)."""
    nn_a = np.asarray(nn_a)
    nn_b = np.asarray(nn_b)
    bad = [np.nonzero(nn_a != nn_b)[0]]
    N = len(nn_a)
    for lo in range(0, N, chunk):
        hi = min(N, lo + chunk)
        ra = padded_sorted_rows(nn_a, nl_a, index_a, lo, hi)
        rb = padded_sorted_rows(nn_b, nl_b, index_b, lo, hi)
        if ra.shape != rb.shape:
            w = max(ra.shape[1], rb.shape[1])
            ra = np.pad(ra, ((0, 0), (0, w - ra.shape[1])), constant_values=PAD)
            rb = np.pad(rb, ((0, 0), (0, w - rb.shape[1])), constant_values=PAD)
        bad.append(lo + np.nonzero((ra != rb).any(axis=1))[0])
    return np.unique(np.concatenate(bad))


def lj_params_dev(par):
    """(ntypes^2, 2) (sigma, epsilon) -> gb_lj_param array at FP32 (EvaluatorPairLJ.h:125-142)."""
    par = np.asarray(par, np.float64).reshape(-1, 2)
    s = par[:, 0].astype(np.float32)
    out = np.zeros((len(par), 2), np.float32)
    out[:, 0] = s * s * s * s * s * s
    out[:, 1] = np.float32(4.0) * par[:, 1].astype(np.float32)
    return dev(out.ravel())


def gpu_pair_forces(nl, kind, params, r_cut, virial=True, shift=0, r_on=None, tables=None, tpp=0):
    """Run one pair kernel through the C ABI; returns (force (N,4), virial (6,N) or None)."""
    L = abi.load()
    rc = np.atleast_2d(np.asarray(r_cut, np.float32))
    rcutsq = dev((rc * rc).ravel())
    ro = np.zeros_like(rc) if r_on is None else np.atleast_2d(np.asarray(r_on, np.float32))
    ronsq = dev((ro * ro).ravel())
    force = zeros(4 * nl.N, torch.float32)
    vir = zeros(6 * nl.N, torch.float32) if virial else None
    a = nl.pair_args(force, vir, rcutsq, ronsq, shift, tpp)
    if kind == "lj":
        d = lj_params_dev(params)
        rc_ = L.gb_pair_forces_lj(ctypes.byref(a), p(d), stream())
    elif kind == "example":
        d = dev(np.asarray(params, np.float32).ravel())
        rc_ = L.gb_pair_forces_example(ctypes.byref(a), p(d), stream())
    else:
        tp, data = tables
        d = dev(np.asarray(tp, np.uint32).ravel())
        td = dev(np.asarray(data, np.float32))
        rc_ = L.gb_pair_forces_table(ctypes.byref(a), p(d), p(td), stream())
    abi.check(rc_, "pair forces")
    f = host(force).reshape(-1, 4)
    v = host(vir).reshape(6, -1) if virial else None
    return f, v


def pack_table(U, F):
    """Packed bins through the C ABI's host helper gb_table_pack: (width, 4) FP32 quads."""
    U = np.ascontiguousarray(U, np.float64)
    F = np.ascontiguousarray(F, np.float64)
    out = np.zeros((len(U), 4), np.float32)
    abi.check(abi.load().gb_table_pack(U.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       F.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       len(U), out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
              "gb_table_pack")
    return out


def table_params(ntypes, tables):
    """tables: {(i, j): (r_min, U, F)} for i <= j -> (gb_table_param records as uint32 words,
    packed FP32 bins, oracle params (ntypes^2, 3), oracle tdata FP64 [U, F] per pair)."""
    recs = np.zeros((ntypes * ntypes, 4), np.uint32)
    data, odata = [], []
    opar = np.zeros((ntypes * ntypes, 3))
    offs, ooffs = {}, {}
    off = ooff = 0
    for (i, j), (rmin, U, F) in sorted(tables.items()):
        offs[(i, j)] = off
        ooffs[(i, j)] = ooff
        data.append(pack_table(U, F).ravel())
        odata.append(np.asarray(U, np.float64))
        odata.append(np.asarray(F, np.float64))
        off += len(U)
        ooff += 2 * len(U)
    for i in range(ntypes):
        for j in range(ntypes):
            a, b = min(i, j), max(i, j)
            rmin, U, F = tables[(a, b)]
            k = i * ntypes + j
            recs[k, 0] = np.float32(rmin).view(np.uint32)
            recs[k, 1] = len(U)
            recs[k, 2] = offs[(a, b)]
            opar[k] = (rmin, len(U), ooffs[(a, b)])
    return recs, np.concatenate(data), opar, np.concatenate(odata)
