"""ctypes binding of the C ABI in include/hoomd_gb300.h (libhoomd_gb300.so).

This is the binding a Python caller (or a HOOMD-blue maintainer wiring the reference's host
classes to these kernels from Python) would write: one ctypes Structure per argument struct and
one prototype per entry point. Device pointers are plain integers (for example
``torch.Tensor.data_ptr()``); ``stream`` is a cudaStream_t as an integer (0 = default stream).
"""

import ctypes
import pathlib
import re

from hoomd_gb300._native import LIB_PATH

c_float, c_uint, c_int, c_u64, c_size, c_void, c_double = (
    ctypes.c_float, ctypes.c_uint32, ctypes.c_int, ctypes.c_uint64, ctypes.c_size_t,
    ctypes.c_void_p, ctypes.c_double)

HEADER = pathlib.Path(__file__).resolve().parents[2] / "include" / "hoomd_gb300.h"

GB_OK, GB_ERR_INVALID, GB_ERR_CUDA, GB_ERR_TOO_LARGE, GB_ERR_UNSUPPORTED = range(5)


class Box(ctypes.Structure):
    _fields_ = [("lo", c_float * 3), ("hi", c_float * 3), ("L", c_float * 3),
                ("Linv", c_float * 3), ("xy", c_float), ("xz", c_float), ("yz", c_float),
                ("periodic", c_uint * 3)]


class CellListArgs(ctypes.Structure):
    _fields_ = [("d_pos", c_void), ("N", c_uint), ("box", Box), ("dim", c_uint * 3),
                ("Nmax", c_uint), ("d_cell_size", c_void), ("d_xyzf", c_void),
                ("d_cell_type", c_void), ("d_conditions", c_void), ("d_gate", c_void),
                ("deterministic", c_int), ("d_build_count", c_void), ("d_timestep", c_void),
                ("d_build_steps", c_void), ("d_dangerous", c_void),
                ("check_delay", ctypes.c_uint32), ("check_dist", c_int),
                ("counts_zeroed", c_int)]


class NlistArgs(ctypes.Structure):
    _fields_ = [("d_nlist", c_void), ("d_n_neigh", c_void), ("d_last_pos", c_void),
                ("d_conditions", c_void), ("d_head_list", c_void), ("stride", c_u64),
                ("interleave", c_uint), ("d_Nmax", c_void), ("d_pos", c_void), ("N", c_uint), ("d_cell_size", c_void),
                ("d_xyzf", c_void), ("d_cell_type", c_void), ("d_cell_adj", c_void),
                ("dim", c_uint * 3), ("Nmax_cell", c_uint), ("adj_width", c_uint), ("box", Box),
                ("d_r_cut", c_void), ("d_r_listsq", c_void), ("ntypes", c_uint),
                ("d_gate", c_void), ("block_size", ctypes.c_uint32), ("nlist_capacity", c_u64),
                ("threads_per_particle", ctypes.c_uint32)]


class PairArgs(ctypes.Structure):
    _fields_ = [("d_force", c_void), ("d_virial", c_void), ("virial_pitch", c_size),
                ("N", c_uint), ("d_pos", c_void), ("d_charge", c_void), ("box", Box),
                ("d_n_neigh", c_void), ("d_nlist", c_void), ("d_head_list", c_void),
                ("stride", c_u64), ("interleave", c_uint), ("d_rcutsq", c_void), ("d_ronsq", c_void), ("ntypes", c_uint),
                ("shift_mode", c_uint), ("compute_virial", c_uint), ("block_size", c_uint),
                ("threads_per_particle", c_uint)]


class StepOneArgs(ctypes.Structure):
    _fields_ = [("d_pos", c_void), ("d_vel", c_void), ("d_accel", c_void), ("d_image", c_void),
                ("N", c_uint), ("box", Box), ("dt", c_float), ("scale", c_float),
                ("d_scale", c_void), ("d_last_pos", c_void), ("d_rcut_max", c_void),
                ("r_buff", c_float), ("d_rebuild", c_void), ("nve_order", c_int),
                ("d_mttk_state", c_void), ("d_mttk_scale2", c_void), ("mttk_dof", c_double),
                ("mttk_kT", c_double), ("mttk_tau", c_double), ("d_mttk_scratch", c_void),
                ("max_displacement", c_float), ("brownian", c_int), ("d_bd_force", c_void),
                ("d_tag", c_void), ("d_gamma", c_void), ("bd_kT", c_float),
                ("ndim", ctypes.c_uint32), ("seed", ctypes.c_uint32), ("d_timestep", c_void),
                ("timestep", c_u64), ("noiseless", c_int), ("d_check_step", c_void),
                ("d_last_update", c_void), ("check_delay", ctypes.c_uint32),
                ("check_dist", c_int), ("d_zero_words", c_void), ("n_zero_words", ctypes.c_uint32)]


class StepFuse(ctypes.Structure):
    _fields_ = [("d_vel", c_void), ("d_accel", c_void), ("dt", c_float), ("d_scale2", c_void),
                ("d_scratch", c_void), ("d_thermo", c_void), ("bussi", c_int), ("dof", c_double),
                ("tau", c_double), ("kT", c_double), ("seed", c_uint), ("instance_id", c_uint),
                ("d_timestep", c_void), ("d_factor", c_void), ("d_status", c_void),
                ("d_rebuild_reset", c_void), ("d_bussi_ring", c_void),
                ("bussi_ring_size", c_uint), ("langevin", c_int), ("d_tag", c_void),
                ("d_pos", c_void), ("d_gamma", c_void), ("langevin_kT", c_float),
                ("ndim", ctypes.c_uint32), ("d_reservoir", c_void), ("berendsen", c_int),
                ("brownian", c_int)]


class EnergySets(ctypes.Structure):
    _fields_ = [("d_mult1", c_void), ("d_mult2", c_void), ("d_n_ex", c_void),
                ("d_ex_list", c_void), ("ex_pitch", c_uint)]


class RadialParam(ctypes.Structure):
    _fields_ = [("v", c_float * 6), ("kind", c_uint), ("aux", c_float)]


class MlpForceArgs(ctypes.Structure):
    _fields_ = [("d_force", c_void), ("d_pos", c_void), ("N", c_uint), ("box", Box),
                ("d_n_neigh", c_void), ("d_nlist", c_void), ("stride", c_u64), ("Nmax", c_uint),
                ("ntypes", c_uint), ("r_min", c_float), ("r_cut", c_float), ("act_split", c_int),
                ("d_infer", c_void), ("d_scratch", c_void), ("mma_sync", c_int)]


_P = ctypes.POINTER
_PROTOS = {
    "gb_box_make": (c_int, [_P(c_double), c_double, c_double, c_double, _P(c_int), _P(Box)]),
    "gb_cell_dims": (c_int, [_P(Box), c_uint, c_float, _P(c_uint)]),
    "gb_last_error": (ctypes.c_char_p, []),
    "gb_version": (c_int, []),
    "gb_cell_list_build": (c_int, [_P(CellListArgs), c_void]),
    "gb_cell_adj_build": (c_int, [_P(c_uint), c_uint, c_void, _P(c_uint), c_void]),
    "gb_nlist_build_binned": (c_int, [_P(NlistArgs), c_void]),
    "gb_nlist_needs_update": (c_int, [c_void, c_void, c_void, c_uint, _P(Box), c_void, c_float,
                                      c_uint, c_float, _P(c_float), c_uint, c_void]),
    "gb_nlist_head_list": (c_int, [c_void, c_void, c_void, c_uint, c_void, c_uint, c_void]),
    "gb_pair_forces_lj": (c_int, [_P(PairArgs), c_void, c_void]),
    "gb_pair_forces_table": (c_int, [_P(PairArgs), c_void, c_void, c_void]),
    "gb_table_pack": (c_int, [_P(c_double), _P(c_double), c_uint, _P(c_float)]),
    "gb_pair_forces_example": (c_int, [_P(PairArgs), c_void, c_void]),
    "gb_cv_step_one": (c_int, [c_void, c_void, c_void, c_void, c_uint, _P(Box), c_float, c_float,
                               c_void, c_void]),
    "gb_cv_step_two": (c_int, [c_void, c_void, c_void, c_uint, c_float, c_float, c_void, c_void]),
    "gb_thermo_scratch_bytes": (c_size, [c_uint]),
    "gb_thermo_reduce": (c_int, [c_void, c_void, c_void, c_size, c_uint, c_void, c_void, c_void]),
    "gb_thermo_reduce_noalloc": (c_int, [c_void, c_void, c_void, c_size, c_uint, c_void, c_void]),
    "gb_bussi_factor": (c_int, [c_void, c_double, c_double, c_double, c_double, c_u64,
                                ctypes.c_uint16, c_uint, c_void, c_void]),
    "gb_bussi_draws": (c_int, [c_void, c_uint, c_double, ctypes.c_uint16, c_uint, c_void, c_uint,
                               c_void]),
    "gb_thermalize": (c_int, [c_void, c_void, c_uint, c_double, c_u64, ctypes.c_uint16, c_uint,
                              c_void, c_void]),
    "gb_graph_set_conditional": (c_int, [c_u64, c_void, c_void]),
    "gb_step_counter_advance": (c_int, [c_void, c_void]),
    "gb_snapshot_stage_bytes": (c_size, [c_uint]),
    "gb_snapshot_gather": (c_int, [c_void, c_void, c_void, c_void, c_uint, c_void, c_void, c_void,
                                   c_void, c_void, c_void]),
    "gb_rtag": (c_int, [c_void, c_uint, c_void, c_void]),
    "gb_snapshot_scatter": (c_int, [c_void, c_void, c_void, c_void, c_void, c_void, c_void, c_uint,
                                    c_uint, _P(Box), c_void, c_void, c_void, c_void, c_void,
                                    c_void, c_void]),
    "gb_md_step_one": (c_int, [_P(StepOneArgs), c_void]),
    "gb_abi_struct_sizes": (c_uint, [_P(c_size), c_uint]),
    "gb_npt_step_one": (c_int, [c_void, c_void, c_void, c_void, c_uint, _P(Box), c_float, c_float,
                                c_void, c_void, c_void, c_void]),
    "gb_npt_step_two": (c_int, [c_void, c_void, c_void, c_uint, c_float, c_float, c_void,
                                c_void]),
    "gb_thermo_tensor_scratch_bytes": (c_size, [c_uint]),
    "gb_thermo_tensor": (c_int, [c_void, c_void, c_void, c_size, c_uint, c_void, c_void, c_void]),
    "gb_berendsen_factor": (c_int, [c_void, c_double, c_double, c_double, c_double, c_void, c_void,
                                    c_void]),
    "gb_normal_draw": (c_int, [ctypes.c_uint8, c_u64, ctypes.c_uint16, ctypes.c_uint32, c_double,
                               c_void, c_void]),
    "gb_langevin_step_two": (c_int, [c_void, c_void, c_void, c_void, c_void, c_void, c_uint,
                                     c_float, c_float, ctypes.c_uint32, ctypes.c_uint16, c_void,
                                     c_void, c_void, c_void, c_void]),
    "gb_md_step_scratch_bytes": (c_size, [c_uint]),
    "gb_md_pair_step_lj": (c_int, [_P(PairArgs), c_void, _P(StepFuse), c_void]),
    "gb_md_pair_step_table": (c_int, [_P(PairArgs), c_void, c_void, _P(StepFuse), c_void]),
    "gb_md_pair_step_example": (c_int, [_P(PairArgs), c_void, _P(StepFuse), c_void]),
    "gb_sum_net_force": (c_int, [c_void, _P(c_void), c_uint, c_uint, c_void]),
    "gb_sfc_scratch_bytes": (c_size, [c_uint, c_int]),
    "gb_sfc_scratch_bytes_dim": (c_size, [c_uint, c_int, c_uint]),
    "gb_sfc_order_dim": (c_int, [c_void, c_uint, _P(Box), c_int, c_uint, c_void, c_void, c_size,
                                 c_void]),
    "gb_sfc_order": (c_int, [c_void, c_uint, _P(Box), c_int, c_void, c_void, c_size, c_void]),
    "gb_gather": (c_int, [c_void, c_void, c_void, c_uint, c_uint, c_void]),
    "gb_pair_forces_radial": (c_int, [c_void, c_void, c_void]),
    "gb_pair_energy_sets_blocks": (c_uint, [c_uint]),
    "gb_pair_energy_sets_lj": (c_int, [c_void, c_void, c_void, c_void, c_void]),
    "gb_pair_energy_sets_table": (c_int, [c_void, c_void, c_void, c_void, c_void, c_void]),
    "gb_pair_energy_sets_example": (c_int, [c_void, c_void, c_void, c_void, c_void]),
    "gb_pair_energy_sets_radial": (c_int, [c_void, c_void, c_void, c_void, c_void]),
    "gb_pair_forces_dpd": (c_int, [c_void, c_void, c_void, c_void, c_int, c_u64, ctypes.c_uint16,
                                   c_float, c_float, c_void]),
    "gb_md_pair_step_radial": (c_int, [c_void, c_void, c_void, c_void]),
    "gb_nlist_filter": (c_int, [c_void, c_void, c_void, c_u64, ctypes.c_uint32, c_uint, c_void,
                                c_void, c_uint, c_void, c_void]),
    "gb_replica_scratch_bytes": (c_size, [ctypes.c_uint64]),
    "gb_replica_smem_bytes": (c_size, [ctypes.c_uint32, ctypes.c_uint32]),
    "gb_replica_ctas_per_sm": (c_int, [ctypes.c_uint32, ctypes.c_uint32]),
    "gb_replicas_run": (c_int, [c_void, c_void]),
    "gb_mlp_param_count": (c_size, [ctypes.c_uint32]),
    "gb_mlp_train_scratch_bytes": (c_size, [ctypes.c_uint32]),
    "gb_mlp_loss_grad": (c_int, [c_void, ctypes.c_uint32, c_float, c_float, c_void, c_void, c_void,
                                 c_void, ctypes.c_uint32, c_float, c_int, c_void, c_void, c_void,
                                 c_void]),
    "gb_mlp_adam": (c_int, [c_void, c_void, c_void, c_void, c_size, c_float, c_float, c_float,
                            c_float, ctypes.c_uint32, c_void]),
    "gb_mlp_infer_bytes": (c_size, [ctypes.c_uint32]),
    "gb_mlp_prepare": (c_int, [c_void, ctypes.c_uint32, c_void, c_void]),
    "gb_mlp_eval": (c_int, [c_void, ctypes.c_uint32, c_float, c_float, c_int, c_void, c_void,
                            ctypes.c_uint32, c_void, c_void, c_void]),
    "gb_mlp_forces_scratch_bytes": (c_size, [c_uint, c_uint]),
    "gb_mlp_forces": (c_int, [c_void, c_void]),
}

_lib = None


def load():
    """Load libhoomd_gb300.so and attach the prototypes."""
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        check_struct_sizes(lib)
        _lib = lib
    return _lib


def check_struct_sizes(lib):
    """Refuse a library whose argument structs differ in size from the mirrors here: a struct
    passed short would have the library read fields past its end."""
    mirrors = [Box, CellListArgs, NlistArgs, PairArgs, RadialParam, StepOneArgs, StepFuse,
               MlpForceArgs]
    sizes = (c_size * 10)()
    lib.gb_abi_struct_sizes(sizes, 10)
    bad = [(m.__name__, ctypes.sizeof(m), sizes[k]) for k, m in enumerate(mirrors)
           if ctypes.sizeof(m) != sizes[k]]
    if bad:
        raise RuntimeError(f"C-ABI struct mirrors differ from the library: {bad}")


def declared_functions(header=HEADER):
    """Names of every function declared in include/hoomd_gb300.h."""
    text = re.sub(r"/\*.*?\*/", "", pathlib.Path(header).read_text(), flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(gb_\w+)\s*\(", text,
                                 flags=re.M)))


def check(rc, what=""):
    if rc != GB_OK:
        msg = load().gb_last_error()
        raise RuntimeError(f"{what}: gb_status {rc}: {msg.decode() if msg else ''}")


def make_box(L, tilts=(0.0, 0.0, 0.0), periodic=(1, 1, 1)):
    b = Box()
    Ld = (c_double * 3)(*[float(x) for x in L])
    per = (c_int * 3)(*[int(p) for p in periodic])
    check(load().gb_box_make(Ld, float(tilts[0]), float(tilts[1]), float(tilts[2]), per,
                             ctypes.byref(b)), "gb_box_make")
    return b


def cell_dims(box, ndim, width):
    d = (c_uint * 3)()
    check(load().gb_cell_dims(ctypes.byref(box), ndim, width, d), "gb_cell_dims")
    return [d[0], d[1], d[2]]
