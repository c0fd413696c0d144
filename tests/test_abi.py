"""CPU checks of the drop-in boundary: the C-ABI library loads, exports every symbol that
include/hoomd_gb300.h declares, and its host-only helpers (box construction, cell-grid
dimensions) round exactly as the reference's BoxDim / CellList do at FP32. No GPU calls."""

import ctypes

import numpy as np
import pytest

from oracle import oracle as O


def test_library_exports_every_declared_symbol():
    from hoomd_gb300 import abi
    names = abi.declared_functions()
    assert len(names) >= 25
    lib = ctypes.CDLL(str(abi.LIB_PATH))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # every declared function has a ctypes prototype in the binding
    assert set(names) <= set(abi._PROTOS), set(names) - set(abi._PROTOS)
    abi.load()


def test_engine_module_imports():
    import hoomd_gb300
    assert hoomd_gb300._hoomd_gb300.version() == 1
    for cls in ("ParticleData", "NeighborListGPUBinned", "PotentialPairGPU", "IntegratorTwoStep"):
        assert hasattr(hoomd_gb300._hoomd_gb300, cls)


def test_every_pair_force_has_its_reference_engine_class():
    """Each md.pair class finds its engine class as the reference's does
    (hoomd/md/pair/pair.py:126-146: _ext_module, _cpp_class_name + "GPU")."""
    import inspect

    from hoomd_gb300.md import pair
    names = []
    for name, cls in vars(pair).items():
        if inspect.isclass(cls) and issubclass(cls, pair.Pair) and cls._cpp_class_name:
            assert hasattr(cls._ext_module, cls._cpp_class_name + "GPU"), name
            names.append(cls._cpp_class_name)
    for ref in ("PotentialPairLJ", "PotentialPairTable", "PotentialPairGauss", "PotentialPairYukawa",
                "PotentialPairEwald", "PotentialPairDPDThermoDPD", "PotentialPairConservativeDPD",
                "PotentialPairLJGauss", "PotentialPairReactionField", "PotentialPairFourier"):
        assert ref in names, ref


@pytest.mark.parametrize("box6", [(16.957, 16.957, 16.957, 0, 0, 0), (10, 11, 12, 0.3, -0.2, 0.1),
                                  (107.67, 107.67, 107.67, 0, 0, 0)])
def test_box_make_matches_oracle_fp32(box6):
    from hoomd_gb300 import abi
    b = abi.make_box(box6[:3], box6[3:])
    L = np.array(b.L[:], np.float32)
    assert np.array_equal(L, np.asarray(box6[:3], np.float32))
    assert np.array_equal(np.array(b.hi[:], np.float32), L / np.float32(2))
    assert np.array_equal(np.array(b.Linv[:], np.float32), np.float32(1) / L)
    # cell dims identical to the oracle's CellList::computeDimensions at FP32
    for w in (2.9, 2.8, 1.1, 3.4, 0.5):
        assert abi.cell_dims(b, 3, w) == O.cell_dims(box6, w, 3, 32).tolist()


def test_c_abi_rejects_bad_arguments_without_gpu():
    from hoomd_gb300 import abi
    lib = abi.load()
    # null arguments are rejected before any CUDA call
    assert lib.gb_cell_list_build(None, None) == abi.GB_ERR_INVALID
    assert b"null" in lib.gb_last_error()
    assert lib.gb_nlist_build_binned(None, None) == abi.GB_ERR_INVALID
    assert lib.gb_pair_forces_lj(None, None, None) == abi.GB_ERR_INVALID
    args = abi.PairArgs()
    args.N = 10
    assert lib.gb_pair_forces_lj(ctypes.byref(args), None, None) == abi.GB_ERR_INVALID
    b = abi.make_box((10, 10, 10))
    assert lib.gb_cell_dims(ctypes.byref(b), 3, 0.0, (ctypes.c_uint32 * 3)()) == abi.GB_ERR_INVALID
    # kernel parameters of the tiled builds are checked before anything runs (the pointers below
    # are never dereferenced)
    fake = ctypes.c_void_p(0x1000)
    nl = abi.NlistArgs(d_nlist=fake, d_n_neigh=fake, d_conditions=fake, d_Nmax=fake,
                       d_cell_size=fake, d_xyzf=fake, d_cell_adj=fake, d_r_cut=fake,
                       d_r_listsq=fake, ntypes=1, N=8, stride=8, adj_width=27)
    for block, tpp in ((96, 0), (128, 2), (128, 16)):
        nl.block_size, nl.threads_per_particle = block, tpp
        assert lib.gb_nlist_build_binned(ctypes.byref(nl), None) == abi.GB_ERR_INVALID
    assert b"threads_per_particle" in lib.gb_last_error()


def test_table_pack_layout():
    """gb_table_pack: bin k = (U[k], F[k], U[k+1], F[k+1]) with zeros past the last point (the
    reference's V1 = F1 = 0 in the last bin, hoomd/md/EvaluatorPairTable.h:172-178)."""
    from gpu_util_cpu import pack_table_cpu
    U = np.array([5.0, 4.0, 3.0, 2.0])
    F = np.array([2.0, 2.5, 3.0, 3.5])
    q = pack_table_cpu(U, F)
    assert q.shape == (4, 4)
    assert np.array_equal(q[0], np.float32([5.0, 2.0, 4.0, 2.5]))
    assert np.array_equal(q[3], np.float32([2.0, 3.5, 0.0, 0.0]))


def test_replica_host_helpers():
    """Host-only sizes of the replica-ensemble launch; no GPU call."""
    from hoomd_gb300 import abi
    lib = abi.load()
    n = 1000
    assert lib.gb_replica_scratch_bytes(n) >= n * (4 + 16) + (n + 31) // 32 * 16
    # double2 Bussi draws per thread, cell starts and counters, 16-byte rounded
    # Bussi draws, cell starts and counters, and per warp the candidate-stream scratch
    assert lib.gb_replica_smem_bytes(1000, 512) == ((512 * 16 + 2001 * 4 + 15) // 16 * 16
                                                    + 16 * (512 + 128 + 2 * 4 * 32 * 12))
    assert lib.gb_replica_smem_bytes(100000, 1024) == 0  # beyond 227 KB of shared memory
    assert lib.gb_replicas_run(None, None) == abi.GB_ERR_INVALID
