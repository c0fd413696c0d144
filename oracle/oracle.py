"""ORACLE -- test infrastructure only.

ctypes front end for the CPU restatement in ``oracle/md_oracle.cc`` (built by ``oracle/build.py``
into ``oracle/_build/``). Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module, and only as the reference the GPU results are compared with or
the timed CPU baseline; the product
package never does.

Precision: every entry point exists at FP32 (``prec=32``, HOOMD built with
``HOOMD_LONGREAL_SIZE=32``) and FP64 (``prec=64``, the reference's default ``Scalar``).
"""

import ctypes
import os
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libmd_oracle.so"

_c_u32p = ctypes.POINTER(ctypes.c_uint32)
_c_u64p = ctypes.POINTER(ctypes.c_uint64)
_c_i32p = ctypes.POINTER(ctypes.c_int32)
_c_f64p = ctypes.POINTER(ctypes.c_double)

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from oracle import build as _b  # noqa: F401  (same directory package)
            _b.build_oracle()
        _lib = ctypes.CDLL(str(LIB_PATH))
        _lib.orc_bussi_factor.restype = ctypes.c_double
        for suf in ("f32", "f64"):
            getattr(_lib, f"orc_kinetic_energy_{suf}").restype = ctypes.c_double
            getattr(_lib, f"orc_langevin_step_two_{suf}").restype = ctypes.c_double
            getattr(_lib, f"orc_sim_reservoir_{suf}").restype = ctypes.c_double
            getattr(_lib, f"orc_sim_create_{suf}").restype = ctypes.c_void_p
            getattr(_lib, f"orc_sim_error_{suf}").restype = ctypes.c_char_p
            for name in ("run", "get", "stats", "destroy", "error"):
                getattr(_lib, f"orc_sim_{name}_{suf}").argtypes = None
        _lib.orc_cell_adj.restype = ctypes.c_uint32
    return _lib


def rdtype(prec):
    return np.float32 if prec == 32 else np.float64


def suf(prec):
    return "f32" if prec == 32 else "f64"


def ptr(a):
    """Raw pointer of a contiguous numpy array (caller keeps the array alive)."""
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


def box6(box):
    b = np.zeros(6, np.float64)
    b[: len(box)] = box
    return b


def periodic3(periodic=(1, 1, 1)):
    return np.asarray(periodic, np.int32)


# --- geometry -------------------------------------------------------------------------------------

def min_image(v, box, prec=32, use_rint=True, periodic=(1, 1, 1)):
    v = np.ascontiguousarray(v, rdtype(prec)).copy()
    b, p = box6(box), periodic3(periodic)
    getattr(lib(), f"orc_min_image_{suf(prec)}")(len(v), ptr(b), ptr(p), ptr(v), int(use_rint))
    return v


def wrap(v, img, box, prec=32, periodic=(1, 1, 1)):
    v = np.ascontiguousarray(v, rdtype(prec)).copy()
    img = np.ascontiguousarray(img, np.int32).copy()
    b, p = box6(box), periodic3(periodic)
    getattr(lib(), f"orc_wrap_{suf(prec)}")(len(v), ptr(b), ptr(p), ptr(v), ptr(img))
    return v, img


def make_fraction(v, box, prec=32, periodic=(1, 1, 1)):
    v = np.ascontiguousarray(v, rdtype(prec)).copy()
    b, p = box6(box), periodic3(periodic)
    getattr(lib(), f"orc_make_fraction_{suf(prec)}")(len(v), ptr(b), ptr(p), ptr(v))
    return v


def nearest_plane_distance(box, prec=32, periodic=(1, 1, 1)):
    out = np.zeros(3, rdtype(prec))
    b, p = box6(box), periodic3(periodic)
    getattr(lib(), f"orc_nearest_plane_distance_{suf(prec)}")(ptr(b), ptr(p), ptr(out))
    return out


# --- evaluators -----------------------------------------------------------------------------------

def _eval(name, prec, rsq, *args):
    rsq = np.ascontiguousarray(rsq, np.float64)
    n = len(rsq)
    f = np.zeros(n, rdtype(prec))
    e = np.zeros(n, rdtype(prec))
    ok = np.zeros(n, np.int32)
    getattr(lib(), f"orc_{name}_eval_{suf(prec)}")(n, ptr(rsq), *args, ptr(f), ptr(e), ptr(ok))
    return f, e, ok.astype(bool)


def lj_eval(rsq, rcutsq, sigma, epsilon, shift=False, prec=32):
    d = ctypes.c_double
    return _eval("lj", prec, rsq, d(rcutsq), d(sigma), d(epsilon), int(shift))


def lj_lrc(rcutsq, sigma, epsilon, prec=32):
    out = np.zeros(2, rdtype(prec))
    d = ctypes.c_double
    getattr(lib(), f"orc_lj_lrc_{suf(prec)}")(d(rcutsq), d(sigma), d(epsilon), ptr(out))
    return out


def table_eval(rsq, rcutsq, rmin, V, F, prec=32):
    V = np.ascontiguousarray(V, rdtype(prec))
    F = np.ascontiguousarray(F, rdtype(prec))
    d = ctypes.c_double
    return _eval("table", prec, rsq, d(rcutsq), d(rmin), len(V), ptr(V), ptr(F))


def example_eval(rsq, rcutsq, k, sigma, shift=False, prec=32):
    d = ctypes.c_double
    return _eval("example", prec, rsq, d(rcutsq), d(k), d(sigma), int(shift))


# --- cell list and neighbour list -----------------------------------------------------------------

def cell_dims(box, nominal_width, ndim=3, prec=32, periodic=(1, 1, 1)):
    out = np.zeros(3, np.uint32)
    b, p = box6(box), periodic3(periodic)
    getattr(lib(), f"orc_cell_dims_{suf(prec)}")(ptr(b), ptr(p), int(ndim),
                                                 ctypes.c_double(nominal_width), ptr(out))
    return out


def cell_adj(dim, ndim=3, radius=1):
    dim = np.ascontiguousarray(dim, np.uint32)
    ncell = int(np.prod(dim))
    adj = np.zeros(27 * ncell, np.uint32)
    w = lib().orc_cell_adj(ptr(dim), int(ndim), int(radius), ptr(adj))
    return adj[: w * ncell].reshape(ncell, w)


def cell_list(pos4, box, dim, Nmax, prec=32, periodic=(1, 1, 1)):
    pos4 = np.ascontiguousarray(pos4, rdtype(prec))
    dim = np.ascontiguousarray(dim, np.uint32)
    ncell = int(np.prod(dim))
    cell_size = np.zeros(ncell, np.uint32)
    xyzf = np.zeros((ncell * Nmax, 4), rdtype(prec))
    cond = np.zeros(3, np.uint32)
    b, p = box6(box), periodic3(periodic)
    getattr(lib(), f"orc_cell_list_{suf(prec)}")(len(pos4), ptr(pos4), ptr(b), ptr(p), ptr(dim),
                                                 int(Nmax), ptr(cell_size), ptr(xyzf), ptr(cond))
    return cell_size, xyzf, cond


def pos_index_bits(w, prec):
    """Decode the particle index or type stored bitwise in the w lane (HOOMD __scalar_as_int)."""
    if prec == 32:
        return np.ascontiguousarray(w, np.float32).view(np.uint32)
    return (np.ascontiguousarray(w, np.float64).view(np.uint64) & 0xFFFFFFFF).astype(np.uint32)


def types_as_w(types, prec):
    t = np.asarray(types, np.uint32)
    if prec == 32:
        return t.view(np.float32)
    return t.astype(np.uint64).view(np.float64)


def make_pos4(xyz, types, prec):
    xyz = np.asarray(xyz)
    pos4 = np.zeros((len(xyz), 4), rdtype(prec))
    pos4[:, :3] = xyz
    pos4[:, 3] = types_as_w(np.asarray(types, np.uint32), prec)
    return pos4


def rlist_matrices(r_cut, r_buff, prec):
    """hoomd/md/NeighborList.cc:452-529 updateRList: r_listsq = (r_cut + r_buff)^2 where r_cut > 0."""
    R = rdtype(prec)
    r_cut = np.asarray(r_cut, R)
    rl = np.where(r_cut > 0, r_cut + R(r_buff), R(0)).astype(R)
    return r_cut, (rl * rl).astype(R)


def build_nlist(pos4, box, r_cut, r_buff, full=True, ndim=3, prec=32, periodic=(1, 1, 1),
                rint_min_image=True, nthreads=1):
    """One neighbour-list build with the overflow retry loops of hoomd/CellList.cc:133-200 and
    hoomd/md/NeighborList.cc:412-427. Returns (n_neigh, nlist, head_list, extra-info dict).
    ``nthreads`` OpenMP threads each build whole particle lists (the result does not depend on
    the thread count)."""
    R = rdtype(prec)
    pos4 = np.ascontiguousarray(pos4, R)
    N = len(pos4)
    r_cut = np.atleast_2d(np.asarray(r_cut, np.float64))
    ntypes = r_cut.shape[0]
    rc, rlsq = rlist_matrices(r_cut, r_buff, prec)
    rc = np.ascontiguousarray(rc.ravel())
    rlsq = np.ascontiguousarray(rlsq.ravel())
    rmax = float(R(rc.max()) + R(r_buff))
    dim = cell_dims(box, rmax, ndim, prec, periodic)
    ncell = int(np.prod(dim))
    Nmax_cell = max(1, int(np.ceil(N / ncell)))
    while True:
        cell_size, xyzf, cond = cell_list(pos4, box, dim, Nmax_cell, prec, periodic)
        if cond[1] or cond[2]:
            raise RuntimeError(f"cell list conditions {cond.tolist()}")
        if cond[0] > Nmax_cell:
            Nmax_cell = int(cond[0])
            continue
        break
    adj = np.ascontiguousarray(cell_adj(dim, ndim, 1))
    types = pos_index_bits(pos4[:, 3], prec)
    Nmax = np.full(ntypes, 4, np.uint32)
    b, p = box6(box), periodic3(periodic)
    while True:
        head = np.zeros(N, np.uint64)
        if N:
            head[1:] = np.cumsum(Nmax[types][:-1].astype(np.uint64))
        total = int(head[-1] + Nmax[types[-1]]) if N else 0
        nlist = np.zeros(max(total, 1), np.uint32)
        n_neigh = np.zeros(N, np.uint32)
        conditions = np.zeros(ntypes, np.uint32)
        getattr(lib(), f"orc_nlist_binned_{suf(prec)}")(
            N, ptr(pos4), ptr(b), ptr(p), ntypes, ptr(rc), ptr(rlsq), int(full), ptr(dim),
            ptr(cell_size), ptr(xyzf), Nmax_cell, ptr(adj), adj.shape[1], ptr(Nmax), ptr(head),
            ptr(nlist), ptr(n_neigh), ptr(conditions), int(rint_min_image), int(nthreads))
        over = conditions > Nmax
        if not over.any():
            break
        Nmax = np.where(over, np.where(conditions > 4, (conditions + 3) & ~np.uint32(3), 4),
                        Nmax).astype(np.uint32)
    info = dict(dim=dim, Nmax_cell=Nmax_cell, cell_size=cell_size, Nmax=Nmax, adj=adj)
    return n_neigh, nlist, head, info


def sfc_order(pos4, box, grid=256, ndim=3, periodic=(1, 1, 1)):
    """hoomd/SFCPackTuner.cc:489-651: the new order (order[new] = old index) of the particle sort
    on a grid^3 Hilbert traversal (grid^2 row-major in 2D), FP32 fractions."""
    pos4 = np.ascontiguousarray(pos4, np.float32)
    N = len(pos4)
    out = np.zeros(N, np.uint32)
    b, p = box6(box), periodic3(periodic)
    lib().orc_sfc_order_f32(N, ptr(pos4), ptr(b), ptr(p), int(grid), int(ndim), ptr(out))
    return out


def neighbor_sets(n_neigh, nlist, head):
    """Per-particle sorted neighbour index arrays."""
    return [np.sort(nlist[int(h): int(h) + int(n)]) for n, h in zip(n_neigh, head)]


def pair_forces(kind, pos4, box, params, rcutsq, n_neigh, nlist, head, third_law=False,
                compute_virial=True, shift_mode=0, ronsq=None, tdata=None, prec=32,
                periodic=(1, 1, 1), rint_min_image=True, nthreads=1, abs_terms=False):
    """hoomd/md/PotentialPair.h:587-794. kind: 'lj' (params ntypes^2 x (sigma, epsilon)),
    'table' (ntypes^2 x (r_min, width, offset) into tdata = concatenated [V, F] per pair),
    'example' (ntypes^2 x (k, sigma)). abs_terms=True (full list only) sums the magnitudes of
    the terms instead: the conditioning of each force, energy and virial sum; abs_terms=2 sums
    the magnitudes of the terms of the pairs within 1e-6 relative of r_cut^2 only (evaluated just
    inside r_cut), the part of each value that two correct FP32 evaluations may include or not."""
    if abs_terms and third_law:
        raise ValueError("abs_terms needs the full list (third_law=False)")
    R = rdtype(prec)
    pos4 = np.ascontiguousarray(pos4, R)
    N = len(pos4)
    kid = {"lj": 0, "table": 1, "example": 2}[kind]
    params = np.ascontiguousarray(params, np.float64).ravel()
    rcutsq = np.ascontiguousarray(rcutsq, R).ravel()
    ronsq = np.zeros_like(rcutsq) if ronsq is None else np.ascontiguousarray(ronsq, R).ravel()
    tdata = np.zeros(1, R) if tdata is None else np.ascontiguousarray(tdata, R)
    ntypes = int(round(np.sqrt(len(rcutsq))))
    force = np.zeros((N, 4), R)
    virial = np.zeros((6, N), R)
    b, p = box6(box), periodic3(periodic)
    n_neigh = np.ascontiguousarray(n_neigh, np.uint32)
    nlist = np.ascontiguousarray(nlist, np.uint32)
    head = np.ascontiguousarray(head, np.uint64)
    getattr(lib(), f"orc_pair_forces_{suf(prec)}")(
        kid, N, ptr(pos4), ptr(b), ptr(p), ntypes, ptr(params), ptr(tdata), ptr(rcutsq),
        ptr(ronsq), int(shift_mode), ptr(n_neigh), ptr(nlist), ptr(head), int(third_law),
        int(compute_virial), ptr(force), ptr(virial), int(rint_min_image), int(nthreads),
        int(abs_terms))
    return force, virial


# --- integrator and thermostat ----------------------------------------------------------------------

def cv_step_one(pos4, vel4, accel3, image3, box, dt, s=1.0, prec=32, periodic=(1, 1, 1)):
    R = rdtype(prec)
    pos4 = np.ascontiguousarray(pos4, R).copy()
    vel4 = np.ascontiguousarray(vel4, R).copy()
    accel3 = np.ascontiguousarray(accel3, R)
    image3 = np.ascontiguousarray(image3, np.int32).copy()
    b, p = box6(box), periodic3(periodic)
    getattr(lib(), f"orc_cv_step_one_{suf(prec)}")(len(pos4), ptr(pos4), ptr(vel4), ptr(accel3),
                                                   ptr(image3), ptr(b), ptr(p),
                                                   ctypes.c_double(dt), ctypes.c_double(s))
    return pos4, vel4, image3


def cv_step_two(vel4, net_force4, dt, s=1.0, prec=32):
    R = rdtype(prec)
    vel4 = np.ascontiguousarray(vel4, R).copy()
    accel3 = np.zeros((len(vel4), 3), R)
    f = np.ascontiguousarray(net_force4, R)
    getattr(lib(), f"orc_cv_step_two_{suf(prec)}")(len(vel4), ptr(vel4), ptr(accel3), ptr(f),
                                                   ctypes.c_double(dt), ctypes.c_double(s))
    return vel4, accel3


def nve_step_one(pos4, vel4, accel3, image3, box, dt, prec=32, periodic=(1, 1, 1)):
    """TwoStepNVE / Langevin step one (x += v dt + a dt^2 / 2, then v += a dt / 2)."""
    R = rdtype(prec)
    pos4 = np.ascontiguousarray(pos4, R).copy()
    vel4 = np.ascontiguousarray(vel4, R).copy()
    accel3 = np.ascontiguousarray(accel3, R)
    image3 = np.ascontiguousarray(image3, np.int32).copy()
    b, p = box6(box), periodic3(periodic)
    getattr(lib(), f"orc_nve_step_one_{suf(prec)}")(len(pos4), ptr(pos4), ptr(vel4), ptr(accel3),
                                                    ptr(image3), ptr(b), ptr(p),
                                                    ctypes.c_double(dt))
    return pos4, vel4, image3


def cv_step_one_capped(pos4, vel4, accel3, image3, box, dt, s, limit, prec=32,
                       periodic=(1, 1, 1)):
    """ConstantVolume step one with the DisplacementCapped limit."""
    R = rdtype(prec)
    pos4 = np.ascontiguousarray(pos4, R).copy()
    vel4 = np.ascontiguousarray(vel4, R).copy()
    accel3 = np.ascontiguousarray(accel3, R)
    image3 = np.ascontiguousarray(image3, np.int32).copy()
    b, p = box6(box), periodic3(periodic)
    d = ctypes.c_double
    getattr(lib(), f"orc_cv_step_one_capped_{suf(prec)}")(
        len(pos4), ptr(pos4), ptr(vel4), ptr(accel3), ptr(image3), ptr(b), ptr(p), d(dt), d(s),
        d(limit))
    return pos4, vel4, image3


def npt_step_one(pos4, vel4, accel3, image3, new_box, dt, s, mv, mr, mri, prec=32,
                 periodic=(1, 1, 1)):
    """ConstantPressure step one with float32 propagators (xx, xy, xz, yy, yz, zz)."""
    R = rdtype(prec)
    pos4 = np.ascontiguousarray(pos4, R).copy()
    vel4 = np.ascontiguousarray(vel4, R).copy()
    accel3 = np.ascontiguousarray(accel3, R)
    image3 = np.ascontiguousarray(image3, np.int32).copy()
    m = [np.ascontiguousarray(x, np.float32) for x in (mv, mr, mri)]
    b, p = box6(new_box), periodic3(periodic)
    getattr(lib(), f"orc_npt_step_one_{suf(prec)}")(
        len(pos4), ptr(pos4), ptr(vel4), ptr(accel3), ptr(image3), ptr(b), ptr(p),
        ctypes.c_double(dt), ctypes.c_double(s), ptr(m[0]), ptr(m[1]), ptr(m[2]))
    return pos4, vel4, image3


def npt_step_two(vel4, net_force4, dt, s, mv, prec=32):
    R = rdtype(prec)
    vel4 = np.ascontiguousarray(vel4, R).copy()
    accel3 = np.zeros((len(vel4), 3), R)
    f = np.ascontiguousarray(net_force4, R)
    m = np.ascontiguousarray(mv, np.float32)
    getattr(lib(), f"orc_npt_step_two_{suf(prec)}")(len(vel4), ptr(vel4), ptr(accel3), ptr(f),
                                                    ctypes.c_double(dt), ctypes.c_double(s),
                                                    ptr(m))
    return vel4, accel3


def bd_step_one(pos4, vel4, force4, image3, tags, gamma, box, kT, dt, seed, timestep, ndim=3,
                noiseless=False, prec=32, periodic=(1, 1, 1)):
    """Brownian (or overdamped, noiseless) step one; returns (pos4, vel4, image3)."""
    R = rdtype(prec)
    pos4 = np.ascontiguousarray(pos4, R).copy()
    vel4 = np.ascontiguousarray(vel4, R).copy()
    f = np.ascontiguousarray(force4, R)
    image3 = np.ascontiguousarray(image3, np.int32).copy()
    tags = np.ascontiguousarray(tags, np.uint32)
    g = np.ascontiguousarray(gamma, np.float64)
    b, p = box6(box), periodic3(periodic)
    getattr(lib(), f"orc_bd_step_one_{suf(prec)}")(
        len(pos4), ptr(pos4), ptr(vel4), ptr(f), ptr(image3), ptr(tags), ptr(g),
        ctypes.c_uint32(len(g)), ptr(b), ptr(p), ctypes.c_double(kT), ctypes.c_double(dt),
        ctypes.c_uint32(seed), ctypes.c_uint64(timestep), ctypes.c_int(ndim),
        ctypes.c_int(int(noiseless)))
    return pos4, vel4, image3


def langevin_step_two(vel4, pos4, tags, net_force4, gamma, kT, dt, seed, timestep, ndim=3,
                      prec=32):
    """Langevin step two; returns (vel4, accel3, sum of F_bd . v)."""
    R = rdtype(prec)
    vel4 = np.ascontiguousarray(vel4, R).copy()
    pos4 = np.ascontiguousarray(pos4, R)
    accel3 = np.zeros((len(vel4), 3), R)
    tags = np.ascontiguousarray(tags, np.uint32)
    f = np.ascontiguousarray(net_force4, R)
    g = np.ascontiguousarray(gamma, np.float64)
    e = getattr(lib(), f"orc_langevin_step_two_{suf(prec)}")(
        len(vel4), ptr(vel4), ptr(accel3), ptr(pos4), ptr(tags), ptr(f), ptr(g),
        ctypes.c_uint32(len(g)), ctypes.c_double(kT), ctypes.c_double(dt), ctypes.c_uint32(seed),
        ctypes.c_uint64(timestep), ctypes.c_int(ndim))
    return vel4, accel3, e


def kinetic_energy(vel4, prec=32):
    vel4 = np.ascontiguousarray(vel4, rdtype(prec))
    return getattr(lib(), f"orc_kinetic_energy_{suf(prec)}")(len(vel4), ptr(vel4))


def thermalize(vel4, tags, kT, timestep, seed, ndim=3, prec=32):
    vel4 = np.ascontiguousarray(vel4, rdtype(prec)).copy()
    tags = np.ascontiguousarray(tags, np.uint32)
    getattr(lib(), f"orc_thermalize_{suf(prec)}")(len(vel4), ptr(vel4), ptr(tags),
                                                  ctypes.c_double(kT), ctypes.c_uint64(timestep),
                                                  int(seed), int(ndim))
    return vel4


def philox(ctr4, key2):
    c = np.ascontiguousarray(ctr4, np.uint32)
    k = np.ascontiguousarray(key2, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(ptr(c), ptr(k), ptr(out))
    return out


def seed_key(rng_id, timestep, seed):
    out = np.zeros(2, np.uint32)
    lib().orc_rng_seed_key(int(rng_id), ctypes.c_uint64(timestep), int(seed), ptr(out))
    return out


def bussi_factor(K, dof, dt, tau, kT, timestep, seed, instance_id):
    d = ctypes.c_double
    return lib().orc_bussi_factor(d(K), d(dof), d(dt), d(tau), d(kT), ctypes.c_uint64(timestep),
                                  int(seed), int(instance_id))


def normal_draws(rng_id, timestep, seed, ctr_a, n):
    out = np.zeros(n, np.float64)
    lib().orc_normal_draws(int(rng_id), ctypes.c_uint64(timestep), int(seed), int(ctr_a), int(n),
                           ptr(out))
    return out


def gamma_draws(rng_id, timestep, seed, ctr_a, alpha, n):
    out = np.zeros(n, np.float64)
    lib().orc_gamma_draws(int(rng_id), ctypes.c_uint64(timestep), int(seed), int(ctr_a),
                          ctypes.c_double(alpha), int(n), ptr(out))
    return out


# --- whole-step runner ------------------------------------------------------------------------------

class Sim:
    """CPU restatement of a HOOMD ConstantVolume (NVE or Bussi) run with one pair force.

    kind 'lj': params = ntypes^2 x (sigma, epsilon); kind 'table': params = ntypes^2 x
    (r_min, width, offset) into tdata. full=False is the reference CPU path (half list, third law);
    full=True is the full-list form, parallel over ``nthreads`` OpenMP threads.
    """

    def __init__(self, pos4, vel4, image3, tags, box, r_cut, r_buff, dt, kind="lj", params=None,
                 tdata=None, shift_mode=0, full=False, bussi=False, kT=1.0, tau=0.0, seed=0,
                 timestep=0, ndim=3, prec=32, nthreads=1, periodic=(1, 1, 1), langevin=None,
                 thermostat=None, mttk_state=(0.0, 0.0)):
        R = rdtype(prec)
        self.prec = prec
        self.N = len(pos4)
        self._keep = []
        pos4 = np.ascontiguousarray(pos4, R)
        vel4 = np.ascontiguousarray(vel4, R)
        image3 = np.ascontiguousarray(image3, np.int32)
        tags = np.ascontiguousarray(tags, np.uint32)
        r_cut = np.ascontiguousarray(np.atleast_2d(r_cut), np.float64).ravel()
        ntypes = int(round(np.sqrt(len(r_cut))))
        params = np.ascontiguousarray(params, np.float64).ravel()
        tdata = np.zeros(1, R) if tdata is None else np.ascontiguousarray(tdata, R)
        b, p = box6(box), periodic3(periodic)
        self._keep = [pos4, vel4, image3, tags, r_cut, params, tdata, b, p]
        d = ctypes.c_double
        self._s = suf(prec)
        L = lib()
        self.h = getattr(L, f"orc_sim_create_{self._s}")(
            ctypes.c_uint32(self.N), ptr(pos4), ptr(vel4), ptr(image3), ptr(tags), ptr(b), ptr(p),
            ctypes.c_int(ndim), ctypes.c_uint32(ntypes), ctypes.c_int({"lj": 0, "table": 1}[kind]),
            ptr(params), ptr(tdata), ctypes.c_size_t(len(tdata)), ptr(r_cut),
            ctypes.c_int(shift_mode), d(r_buff), ctypes.c_int(int(full)), d(dt),
            ctypes.c_int(int(bussi)), d(kT), d(tau), ctypes.c_uint32(seed),
            ctypes.c_uint64(timestep), ctypes.c_int(nthreads))
        self.h = ctypes.c_void_p(self.h)
        if thermostat is not None:
            # "berendsen" or "mttk" with kT and tau (ConstantVolume thermostats)
            kind = {"bussi": 1, "berendsen": 2, "mttk": 3}[thermostat]
            getattr(L, f"orc_sim_set_thermostat_{self._s}")(self.h, ctypes.c_int(kind), d(kT),
                                                             d(tau), d(mttk_state[0]),
                                                             d(mttk_state[1]))
        if langevin is not None:
            # langevin = per-type drag coefficients; kT is the bath temperature
            g = np.ascontiguousarray(langevin, np.float64)
            self._keep.append(g)
            getattr(L, f"orc_sim_set_langevin_{self._s}")(self.h, d(kT), ptr(g))

    def set_thermostat(self, thermostat, kT=1.0, tau=0.0):
        """Replace the ConstantVolume thermostat: None (NVE), "bussi", "berendsen" or "mttk"."""
        kind = {None: 0, "bussi": 1, "berendsen": 2, "mttk": 3}[thermostat]
        getattr(lib(), f"orc_sim_set_thermostat_{self._s}")(
            self.h, ctypes.c_int(kind), ctypes.c_double(kT), ctypes.c_double(tau),
            ctypes.c_double(0.0), ctypes.c_double(0.0))

    @property
    def mttk_state(self):
        out = np.zeros(2, np.float64)
        getattr(lib(), f"orc_sim_mttk_{self._s}")(self.h, ptr(out))
        return tuple(out)

    @property
    def reservoir_energy(self):
        return getattr(lib(), f"orc_sim_reservoir_{self._s}")(self.h)

    def run(self, nsteps):
        rc = getattr(lib(), f"orc_sim_run_{self._s}")(self.h, ctypes.c_uint64(nsteps))
        if rc != 0:
            msg = getattr(lib(), f"orc_sim_error_{self._s}")(self.h)
            raise RuntimeError(ctypes.string_at(msg).decode() if isinstance(msg, int) else msg)

    def get(self):
        R = rdtype(self.prec)
        pos = np.zeros((self.N, 4), R)
        vel = np.zeros((self.N, 4), R)
        img = np.zeros((self.N, 3), np.int32)
        force = np.zeros((self.N, 4), R)
        accel = np.zeros((self.N, 3), R)
        getattr(lib(), f"orc_sim_get_{self._s}")(self.h, ptr(pos), ptr(vel), ptr(img), ptr(force),
                                                 ptr(accel))
        return dict(pos=pos, vel=vel, image=img, force=force, accel=accel)

    def set_check(self, rebuild_check_delay=1, check_dist=True):
        """The neighbour list's rebuild-check schedule (nlist rebuild_check_delay, check_dist)."""
        getattr(lib(), f"orc_sim_set_check_{self._s}")(self.h, ctypes.c_uint(rebuild_check_delay),
                                                        ctypes.c_int(int(check_dist)))

    def stats(self):
        """n_builds counts every build, forced ones included; checked_builds only those a check
        decided (the reference's num_builds), dangerous_builds those at the first check after a
        delay > 1; last_update is the step of the last build."""
        out = np.zeros(8, np.float64)
        getattr(lib(), f"orc_sim_stats_{self._s}")(self.h, ptr(out))
        return dict(timestep=int(out[0]), n_builds=int(out[1]), sum_n_neigh=out[2],
                    kinetic_energy=out[3], potential_energy=out[4], checked_builds=int(out[5]),
                    dangerous_builds=int(out[6]), last_update=int(out[7]))

    def __del__(self):
        try:
            getattr(lib(), f"orc_sim_destroy_{self._s}")(self.h)
        except Exception:
            pass
