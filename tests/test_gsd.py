"""GSD files (hoomd_gb300.gsd, hoomd_gb300.write.GSD): the file layer against the reference's own
GSD library (hoomd/extern/gsd.c built into the oracle's reference directory) in both directions,
the reference-written example file sphinx-doc/howto/spheres.gsd, and the hoomd-schema rules of
GSDDumpWriter / GSDReader (defaults, frame-0 fall-back, dynamic quantities). CPU only."""

import pathlib

import numpy as np
import pytest

from hoomd_gb300.gsd import fl
from hoomd_gb300.gsd import hoomd as gh
from hoomd_gb300.snapshot import Snapshot
from hoomd_gb300 import write as gwrite
from oracle.build import REF_ROOT

try:
    from oracle import gsd_ref
    HAVE_REF = gsd_ref.available()
except Exception:  # pragma: no cover - the reference tree is absent
    HAVE_REF = False

needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference GSD library not built here")
SPHERES = REF_ROOT / "sphinx-doc" / "howto" / "spheres.gsd"

DTYPES = [np.uint8, np.uint16, np.uint32, np.uint64, np.int8, np.int16, np.int32, np.int64,
          np.float32, np.float64]


def random_frames(rng, nframes=6, nnames=5, long_names=False):
    """Frames of chunks with every element type, 1-D and 2-D, some empty, names reused."""
    frames = []
    for f in range(nframes):
        chunks = {}
        for k in range(nnames):
            name = f"group{k % 3}/" + ("q" * 50 if long_names else "q") + f"{k}_{f % 4}"
            dt = DTYPES[(f * nnames + k) % len(DTYPES)]
            N = int(rng.integers(0, 7))
            M = int(rng.integers(1, 4))
            a = (rng.random((N, M)) * 100).astype(dt)
            chunks[name] = a if M > 1 else a.reshape(N)
        frames.append(chunks)
    return frames


def write_own(path, frames, mode="w"):
    with fl.open(path, mode, application="test", schema="test", schema_version=(3, 7)) as f:
        for chunks in frames:
            for name, a in chunks.items():
                f.write_chunk(name, a)
            f.end_frame()


def check_equal(a, b):
    assert a.dtype == b.dtype
    assert a.shape == b.shape
    assert np.array_equal(a, b)


def test_round_trip_own(tmp_path):
    rng = np.random.default_rng(1)
    frames = random_frames(rng)
    p = tmp_path / "a.gsd"
    write_own(p, frames)
    with fl.open(p) as f:
        assert f.nframes == len(frames)
        assert f.gsd_version == (2, 0)
        assert (f.application, f.schema, f.schema_version) == ("test", "test", (3, 7))
        for i, chunks in enumerate(frames):
            for name, a in chunks.items():
                assert f.chunk_exists(i, name)
                check_equal(f.read_chunk(i, name), a)
        assert not f.chunk_exists(0, "missing")
        with pytest.raises(KeyError):
            f.read_chunk(0, "missing")
        with pytest.raises(IndexError):
            f.read_chunk(len(frames), next(iter(frames[0])))


def test_append_truncate_and_modes(tmp_path):
    rng = np.random.default_rng(2)
    frames = random_frames(rng, nframes=4)
    p = tmp_path / "b.gsd"
    write_own(p, frames[:2])
    write_own(p, frames[2:], mode="a")
    with fl.open(p) as f:
        assert f.nframes == 4
        for i, chunks in enumerate(frames):
            for name, a in chunks.items():
                check_equal(f.read_chunk(i, name), a)
    with pytest.raises(FileExistsError):
        fl.open(p, "x", application="t", schema="t", schema_version=(1, 0))
    with fl.open(p, "r+") as f:
        f.truncate()
        assert f.nframes == 0 and f.schema == "test" and f.schema_version == (3, 7)
    with fl.open(p) as f:
        assert f.nframes == 0
    with fl.open(p, "r") as f:
        with pytest.raises(RuntimeError):
            f.write_chunk("x", np.zeros(1))


def test_rejects_bad_input(tmp_path):
    p = tmp_path / "c.gsd"
    p.write_bytes(b"not a gsd file" * 40)
    with pytest.raises(RuntimeError):
        fl.open(p)
    with fl.open(tmp_path / "d.gsd", "w", application="t", schema="t", schema_version=(1, 0)) as f:
        with pytest.raises(ValueError):
            f.write_chunk("x", np.zeros((2, 2, 2)))
        with pytest.raises(ValueError):
            f.write_chunk("x", np.array(["a"]))
        with pytest.raises(ValueError):
            f.write_chunk("x", np.zeros(3, np.complex64))
    # a truncated file (index past the end)
    write_own(tmp_path / "e.gsd", random_frames(np.random.default_rng(3), nframes=2))
    data = (tmp_path / "e.gsd").read_bytes()
    (tmp_path / "f.gsd").write_bytes(data[:600])
    with pytest.raises(RuntimeError):
        fl.open(tmp_path / "f.gsd")


@needs_ref
@pytest.mark.parametrize("many", [False, True])
def test_reference_reads_own_files(tmp_path, many):
    """Files written here are read chunk for chunk by the reference's gsd.c, including files
    whose index (over 128 entries) and name list (over 1024 bytes) had to grow and move."""
    rng = np.random.default_rng(4)
    frames = random_frames(rng, nframes=60 if many else 3, nnames=6, long_names=many)
    p = tmp_path / "own.gsd"
    write_own(p, frames)
    with gsd_ref.RefGSD(p) as r, fl.open(p) as f:
        h = r.header()
        assert h == dict(gsd_version=(2, 0), schema_version=(3, 7), application="test",
                         schema="test")
        assert r.nframes == len(frames)
        assert r.names() == f.find_matching_chunk_names("")
        for i, chunks in enumerate(frames):
            for name, a in chunks.items():
                got = r.read(i, name)
                check_equal(got, a.reshape(got.shape))
    if many:
        assert len(frames) * 6 > fl.INITIAL_INDEX_ENTRIES
        assert sum(len(n) + 1 for n in r_names(p)) > fl.INITIAL_NAMELIST_BYTES


def r_names(p):
    with fl.open(p) as f:
        return f.find_matching_chunk_names("")


@needs_ref
@pytest.mark.parametrize("many", [False, True])
def test_own_reader_reads_reference_files(tmp_path, many):
    rng = np.random.default_rng(5)
    frames = random_frames(rng, nframes=60 if many else 3, nnames=6, long_names=many)
    p = tmp_path / "ref.gsd"
    with gsd_ref.RefGSD(p, "w", application="refapp", schema="hoomd", version=(1, 4)) as r:
        for chunks in frames:
            for name, a in chunks.items():
                r.write(name, a)
            r.end_frame()
    with fl.open(p) as f:
        assert (f.application, f.schema, f.schema_version, f.gsd_version) == \
            ("refapp", "hoomd", (1, 4), (2, 0))
        assert f.nframes == len(frames)
        for i, chunks in enumerate(frames):
            for name, a in chunks.items():
                check_equal(f.read_chunk(i, name), a)


@needs_ref
def test_mixed_appends(tmp_path):
    """The reference appends to a file made here, then this reader appends to that, and both
    libraries read every frame."""
    rng = np.random.default_rng(6)
    frames = random_frames(rng, nframes=30, nnames=6, long_names=True)
    p = tmp_path / "mix.gsd"
    write_own(p, frames[:10])
    with gsd_ref.RefGSD(p, "a") as r:
        for chunks in frames[10:20]:
            for name, a in chunks.items():
                r.write(name, a)
            r.end_frame()
    write_own(p, frames[20:], mode="a")
    with gsd_ref.RefGSD(p) as r, fl.open(p) as f:
        assert r.nframes == f.nframes == 30
        for i, chunks in enumerate(frames):
            for name, a in chunks.items():
                check_equal(f.read_chunk(i, name), a)
                got = r.read(i, name)
                check_equal(got, a.reshape(got.shape))


@needs_ref
@pytest.mark.skipif(not SPHERES.exists(), reason="reference example file absent")
def test_reference_example_file():
    """sphinx-doc/howto/spheres.gsd, written by HOOMD-blue itself: every chunk equal to what the
    reference library reads, and the schema layer's frame."""
    with gsd_ref.RefGSD(SPHERES) as r, fl.open(SPHERES) as f:
        assert r.header()["application"] == f.application
        assert r.nframes == f.nframes
        names = r.names()
        assert names == f.find_matching_chunk_names("")
        for i in range(f.nframes):
            for n in names:
                if r.find(i, n) is None:
                    assert not f.chunk_exists(i, n)
                    continue
                got = r.read(i, n)
                check_equal(f.read_chunk(i, n), got)
    with gh.open(SPHERES) as t:
        fr = t[-1]
        N = fr.particles.N
        with gsd_ref.RefGSD(SPHERES) as r:
            assert np.array_equal(fr.particles.position, r.read(0, "particles/position"))
        assert fr.particles.types == ["A"]
        assert np.array_equal(fr.particles.mass, np.ones(N, np.float32))
        assert np.array_equal(fr.particles.body, np.full(N, -1, np.int32))
        snap = Snapshot.from_gsd_frame(fr)
        snap.validate()
        L = snap.configuration.box[0]
        assert np.all(np.abs(snap.particles.position) <= L / 2)


def make_snapshot(N=20, seed=0):
    rng = np.random.default_rng(seed)
    s = Snapshot()
    s.configuration.box = [8, 8, 8, 0, 0, 0]
    s.particles.N = N
    s.particles.types = ["A", "Bb"]
    s.particles.position[:] = rng.uniform(-4, 4, (N, 3))
    s.particles.velocity[:] = rng.normal(size=(N, 3))
    s.particles.typeid[:] = rng.integers(0, 2, N)
    s.particles.mass[:] = rng.uniform(0.5, 2, N)
    s.particles.image[:] = rng.integers(-2, 3, (N, 3))
    s.particles.charge[:] = rng.normal(size=N)
    s.bonds.N = 3
    s.bonds.types = ["b"]
    s.bonds.group[:] = [[0, 1], [1, 2], [5, 6]]
    s.constraints.N = 1
    s.constraints.value[:] = [1.25]
    s.constraints.group[:] = [[3, 4]]
    return s


def write_frames(path, snaps, steps, dynamic=("property",), mode="wb"):
    with gwrite._open(path, mode) as f:
        nd = gwrite._nondefault(f)
        for s, t in zip(snaps, steps):
            gwrite._write_frame(f, s, t, list(dynamic), nd, False, None)


def test_writer_schema_rules(tmp_path):
    """Frame 0 holds the non-default quantities; later frames the step and the dynamic
    'property' quantities; readers fall back to frame 0 for the rest."""
    s0 = make_snapshot()
    s1 = make_snapshot()
    s1.particles.position[:] *= 0.5
    s1.particles.velocity[:] = 0.0  # not dynamic: stays at frame 0's values when read back
    p = tmp_path / "w.gsd"
    write_frames(p, [s0, s1], [100, 200])
    with fl.open(p) as f:
        assert f.schema == "hoomd" and f.schema_version == (1, 4)
        f0 = set(n for n in f.find_matching_chunk_names("") if f.chunk_exists(0, n))
        f1 = set(n for n in f.find_matching_chunk_names("") if f.chunk_exists(1, n))
        assert {"configuration/step", "configuration/dimensions", "configuration/box",
                "particles/N", "particles/types", "particles/typeid", "particles/mass",
                "particles/charge", "particles/position", "particles/velocity",
                "particles/image", "bonds/N", "bonds/types", "bonds/typeid", "bonds/group",
                "constraints/N", "constraints/value", "constraints/group"} == f0
        assert f1 == {"configuration/step", "configuration/box", "particles/N",
                      "particles/position"}
    with gh.open(p) as t:
        a, b = t[0], t[1]
        assert (a.configuration.step, b.configuration.step) == (100, 200)
        assert np.array_equal(b.particles.position, s1.particles.position.astype(np.float32))
        assert np.array_equal(b.particles.velocity, s0.particles.velocity.astype(np.float32))
        assert np.array_equal(b.particles.charge, s0.particles.charge.astype(np.float32))
        assert b.particles.types == ["A", "Bb"]
        assert np.array_equal(b.bonds.group, s0.bonds.group)
        assert np.allclose(b.constraints.value, [1.25])
        back = Snapshot.from_gsd_frame(b)
        back.validate()
        assert np.array_equal(back.particles.image, s0.particles.image)
        assert np.array_equal(back.particles.orientation, np.tile([1.0, 0, 0, 0], (20, 1)))


def test_writer_default_rule_keeps_frame0_fallback_correct(tmp_path):
    """A dynamic quantity that is all default in a later frame is still written when frame 0
    stored a non-default value (else a reader would take frame 0's), and skipped otherwise."""
    s0 = make_snapshot()
    s0.particles.velocity[:] = 0.0
    s1 = make_snapshot()
    s1.particles.image[:] = 0
    s1.particles.velocity[:] = 0.0
    p = tmp_path / "d.gsd"
    write_frames(p, [s0, s1], [0, 1], dynamic=("property", "momentum"))
    with fl.open(p) as f:
        assert not f.chunk_exists(0, "particles/velocity")
        assert not f.chunk_exists(1, "particles/velocity")
        assert f.chunk_exists(0, "particles/image") and f.chunk_exists(1, "particles/image")
        assert np.array_equal(f.read_chunk(1, "particles/image"), np.zeros((20, 3), np.int32))
    with gh.open(p) as t:
        assert np.array_equal(t[1].particles.image, np.zeros((20, 3), np.int32))


def test_append_mode_reads_nondefault_map(tmp_path):
    s0 = make_snapshot()
    p = tmp_path / "ap.gsd"
    write_frames(p, [s0], [0])
    s1 = make_snapshot()
    s1.particles.image[:] = 0
    write_frames(p, [s1], [5], dynamic=("momentum",), mode="ab")
    with gh.open(p) as t:
        assert len(t) == 2
        assert np.array_equal(t[1].particles.image, np.zeros((20, 3), np.int32))
        assert t[1].configuration.step == 5


def test_positions_are_wrapped_with_images(tmp_path):
    s = make_snapshot(N=4)
    s.particles.position[:] = [[4.5, 0, 0], [-4.5, 0, 0], [0, 12.5, 0], [1, 1, -4.01]]
    s.particles.image[:] = 0
    p = tmp_path / "wrap.gsd"
    write_frames(p, [s], [0])
    with gh.open(p) as t:
        fr = t[0]
        assert np.allclose(fr.particles.position,
                           [[-3.5, 0, 0], [3.5, 0, 0], [0, -3.5, 0], [1, 1, 3.99]], atol=1e-6)
        assert np.array_equal(fr.particles.image, [[1, 0, 0], [-1, 0, 0], [0, 2, 0], [0, 0, -1]])


def test_schema_defaults_and_particle_count_rule(tmp_path):
    """A file with only N and positions reads with the schema defaults; a frame-0 chunk whose
    length differs from the frame's N is not used (hoomd/GSDReader.cc:103-118)."""
    p = tmp_path / "n.gsd"
    with fl.open(p, "w", application="t", schema="hoomd", schema_version=(1, 4)) as f:
        f.write_chunk("particles/N", np.array([3], np.uint32))
        f.write_chunk("particles/mass", np.array([2.0, 3.0, 4.0], np.float32))
        f.end_frame()
        f.write_chunk("particles/N", np.array([2], np.uint32))
        f.end_frame()
    with gh.open(p) as t:
        a, b = t[0], t[1]
        assert a.configuration.dimensions == 3
        assert np.array_equal(a.configuration.box, np.array([1, 1, 1, 0, 0, 0], np.float32))
        assert a.particles.types == ["A"]
        assert np.array_equal(a.particles.mass, [2, 3, 4])
        assert np.array_equal(b.particles.mass, [1, 1])
        assert np.array_equal(b.particles.diameter, [1, 1])
        assert np.array_equal(b.particles.orientation, [[1, 0, 0, 0]] * 2)


def test_trajectory_append_round_trip(tmp_path):
    p = tmp_path / "traj.gsd"
    rng = np.random.default_rng(8)
    written = []
    with gh.open(p, "w") as t:
        for k in range(4):
            fr = gh.Frame()
            fr.configuration.step = 10 * k
            fr.configuration.box = [5, 6, 7, 0.1, 0, 0]
            fr.particles.N = 5
            fr.particles.types = ["A", "B"]
            fr.particles.typeid = [0, 1, 1, 0, 1]
            fr.particles.position = rng.random((5, 3)).astype(np.float32)
            fr.log["md/compute/ThermodynamicQuantities/kinetic_energy"] = np.array([k * 0.5])
            t.append(fr)
            written.append(fr)
    with gh.open(p) as t:
        assert len(t) == 4
        for fr, w in zip(t, written):
            assert fr.configuration.step == w.configuration.step
            assert np.array_equal(fr.configuration.box, w.configuration.box)
            assert np.array_equal(fr.particles.position, w.particles.position)
            assert np.array_equal(fr.particles.typeid, w.particles.typeid)
            assert fr.log == {k: v for k, v in fr.log.items()}
        assert t[-1].log["md/compute/ThermodynamicQuantities/kinetic_energy"][0] == 1.5
        assert [f.configuration.step for f in t[1:3]] == [10, 20]


def test_logger_chunks(tmp_path):
    from hoomd_gb300.logging import Logger

    class Thing:
        _loggables = {"energy": "scalar", "forces": "particle", "label": "string",
                      "obj": "object"}
        _log_namespace = ("md", "pair", "Thing")
        energy = 1.5
        forces = np.ones((20, 3))
        label = "abc"
        obj = object()

    lg = Logger()
    lg.add(Thing())
    lg[("custom", "value")] = (lambda: 7, "scalar")
    assert ("md", "pair", "Thing", "energy") in lg
    nested = lg.log()
    assert nested["md"]["pair"]["Thing"]["energy"] == (1.5, "scalar")
    s = make_snapshot()
    p = tmp_path / "log.gsd"
    with gwrite._open(p, "wb") as f:
        gwrite._write_frame(f, s, 0, ["property"], {}, False, lg)
    with gh.open(p) as t:
        log = t[0].log
        assert log["md/pair/Thing/energy"][0] == 1.5
        assert log["md/pair/Thing/forces"].shape == (20, 3)
        assert bytes(log["md/pair/Thing/label"]).rstrip(b"\0") == b"abc"
        assert log["custom/value"][0] == 7
        assert "md/pair/Thing/obj" not in log
    with pytest.raises(ValueError):
        Logger(categories=["scalar"]).add(Thing(), quantities=["forces"])


def test_surrogate_training_frames_from_gsd(tmp_path):
    from hoomd_gb300.surrogate import gsd_frames
    s = make_snapshot()
    p = tmp_path / "train.gsd"
    s1 = make_snapshot(seed=1)
    write_frames(p, [s, s1], [0, 10], dynamic=("property", "attribute"))
    frames = gsd_frames(p)
    assert len(frames) == 2
    pos, typeid, L = frames[1]
    assert np.array_equal(pos, s1.particles.position.astype(np.float32).astype(np.float64))
    assert np.array_equal(typeid, s1.particles.typeid)
    assert np.array_equal(L, [8, 8, 8])
