"""GSD file layer: chunked, frame-indexed binary files (the GSD 2.0 file layout).

HOOMD-blue reads and writes GSD through its vendored C library (hoomd/extern/gsd.c, gsd.h) and the
``gsd`` Python package (``gsd.fl``). Neither is needed here: this module is an own implementation
of the published file layout, with the ``gsd.fl.GSDFile`` interface (open modes, ``nframes``,
``read_chunk``, ``chunk_exists``, ``write_chunk``, ``end_frame``, ``find_matching_chunk_names``,
``truncate``).

Layout (all integers little endian):

* a 256-byte header at offset 0: magic ``0x65DF65DF65DF65DF``, the location and capacity (in
  entries) of the chunk index, the location and capacity (in 64-byte units) of the name list,
  the schema version and the file-format version (both ``major << 16 | minor``), the application
  and schema names (64 bytes each, NUL terminated) and 80 reserved bytes (hoomd/extern/gsd.h:126);
* the chunk index: 32-byte entries (frame, N, location, M, name id, type, flags) sorted by
  (frame, name id); unused entries are zero, and the first entry with location 0 ends the used
  part (hoomd/extern/gsd.h:165, gsd.c:599-700);
* the name list: NUL-terminated chunk names packed one after another, zero padded; a name's id is
  its position in the list (gsd.c:1276-1320, 1500-1530). Format 1.x files kept one 64-byte slot
  per name; they are read, not appended to;
* the chunk data, ``N x M`` elements of one of ten numeric types, anywhere after the header.

A frame is committed by ``end_frame``: its chunks' data are appended to the file, new names are
added to the name list (which moves to the end of the file, doubled, when it is full), the index
entries are appended (the index moves to the end of the file, doubled, when it is full) and the
header is rewritten. The number of frames is one more than the frame of the last index entry.
"""

import os

import numpy as np

MAGIC = 0x65DF65DF65DF65DF
NAME_SIZE = 64
INITIAL_INDEX_ENTRIES = 128
INITIAL_NAMELIST_BYTES = 1024

HEADER_DTYPE = np.dtype([
    ("magic", "<u8"), ("index_location", "<u8"), ("index_allocated_entries", "<u8"),
    ("namelist_location", "<u8"), ("namelist_allocated_entries", "<u8"),
    ("schema_version", "<u4"), ("gsd_version", "<u4"),
    ("application", "S64"), ("schema", "S64"), ("reserved", "S80")])
INDEX_DTYPE = np.dtype([
    ("frame", "<u8"), ("N", "<u8"), ("location", "<i8"), ("M", "<u4"), ("id", "<u2"),
    ("type", "u1"), ("flags", "u1")])
assert HEADER_DTYPE.itemsize == 256 and INDEX_DTYPE.itemsize == 32

# element type codes of the format (hoomd/extern/gsd.h:22-52)
TYPE_CODES = {1: np.dtype("<u1"), 2: np.dtype("<u2"), 3: np.dtype("<u4"), 4: np.dtype("<u8"),
              5: np.dtype("<i1"), 6: np.dtype("<i2"), 7: np.dtype("<i4"), 8: np.dtype("<i8"),
              9: np.dtype("<f4"), 10: np.dtype("<f8")}
_CODE_OF = {(dt.kind, dt.itemsize): code for code, dt in TYPE_CODES.items()}


def make_version(major, minor):
    return (int(major) << 16) | int(minor)


def split_version(v):
    return (int(v) >> 16, int(v) & 0xFFFF)


def _type_code(dtype):
    dt = np.dtype(dtype)
    code = _CODE_OF.get((dt.kind, dt.itemsize))
    if code is None:
        raise ValueError(f"GSD cannot store arrays of type {dt}")
    return code


class GSDFile:
    """An open GSD file (gsd.fl.GSDFile).

    ``mode``: ``'r'`` read only; ``'r+'`` read and append; ``'w'`` create or overwrite; ``'x'``
    create, failing if the file exists; ``'a'`` append, creating the file when it does not exist.
    The binary spellings ``'rb'``, ``'rb+'``, ``'wb'``, ``'wb+'``, ``'xb'``, ``'xb+'``, ``'ab'``
    are accepted too. Creating a file needs ``application``, ``schema`` and ``schema_version``
    (a ``(major, minor)`` tuple).
    """

    _MODES = {"r": "r", "rb": "r", "r+": "r+", "rb+": "r+", "w": "w", "wb": "w", "wb+": "w",
              "w+": "w", "x": "x", "xb": "x", "xb+": "x", "x+": "x", "a": "a", "ab": "a"}

    def __init__(self, name, mode="r", application=None, schema=None, schema_version=None):
        if mode not in self._MODES:
            raise ValueError(f"invalid GSD file mode {mode!r}")
        self._name = os.fspath(name)
        self._mode = mode
        m = self._MODES[mode]
        self._writable = m != "r"
        self._fd = None
        create = m in ("w", "x") or (m == "a" and not os.path.exists(self._name))
        if create:
            if application is None or schema is None or schema_version is None:
                raise ValueError("creating a GSD file needs application, schema and "
                                 "schema_version")
            flags = os.O_RDWR | os.O_CREAT | (os.O_EXCL if m == "x" else os.O_TRUNC)
            self._fd = os.open(self._name, flags, 0o666)
            self._initialize(str(application), str(schema), tuple(schema_version))
        else:
            self._fd = os.open(self._name, os.O_RDWR if self._writable else os.O_RDONLY)
        try:
            self._load()
        except Exception:
            os.close(self._fd)
            self._fd = None
            raise
        self._pending = []  # (name, array, type code) of the frame being written

    # -- low-level I/O ------------------------------------------------------------------------
    def _pwrite(self, data, offset):
        mv = memoryview(data).cast("B")
        done = 0
        while done < len(mv):
            n = os.pwrite(self._fd, mv[done:], offset + done)
            if n <= 0:
                raise OSError(f"GSD: short write to {self._name}")
            done += n

    def _pread(self, size, offset):
        parts = []
        got = 0
        while got < size:
            b = os.pread(self._fd, size - got, offset + got)
            if not b:
                raise OSError(f"GSD: unexpected end of file in {self._name}")
            parts.append(b)
            got += len(b)
        return b"".join(parts)

    def _initialize(self, application, schema, schema_version):
        os.ftruncate(self._fd, 0)
        h = np.zeros(1, HEADER_DTYPE)
        h["magic"] = MAGIC
        h["gsd_version"] = make_version(2, 0)
        h["application"] = application.encode()[:NAME_SIZE - 1]
        h["schema"] = schema.encode()[:NAME_SIZE - 1]
        h["schema_version"] = make_version(*schema_version)
        h["index_location"] = HEADER_DTYPE.itemsize
        h["index_allocated_entries"] = INITIAL_INDEX_ENTRIES
        h["namelist_location"] = HEADER_DTYPE.itemsize + INDEX_DTYPE.itemsize * INITIAL_INDEX_ENTRIES
        h["namelist_allocated_entries"] = INITIAL_NAMELIST_BYTES // NAME_SIZE
        self._pwrite(h.tobytes(), 0)
        self._pwrite(bytes(INDEX_DTYPE.itemsize * INITIAL_INDEX_ENTRIES), HEADER_DTYPE.itemsize)
        self._pwrite(bytes(INITIAL_NAMELIST_BYTES), int(h["namelist_location"][0]))
        os.fsync(self._fd)

    def _load(self):
        self._file_size = os.fstat(self._fd).st_size
        if self._file_size < HEADER_DTYPE.itemsize:
            raise RuntimeError(f"{self._name} is not a GSD file")
        h = np.frombuffer(self._pread(HEADER_DTYPE.itemsize, 0), HEADER_DTYPE).copy()
        if int(h["magic"][0]) != MAGIC:
            raise RuntimeError(f"{self._name} is not a GSD file")
        version = int(h["gsd_version"][0])
        if not (make_version(1, 0) <= version < make_version(3, 0) or version == make_version(0, 3)):
            raise RuntimeError(f"{self._name}: unsupported GSD file version "
                               f"{split_version(version)}")
        if self._writable and version < make_version(2, 0):
            raise RuntimeError(f"{self._name}: appending to a GSD {split_version(version)} file "
                               "is not supported; open it read only")
        self._header = h
        # name list
        nbytes = NAME_SIZE * int(h["namelist_allocated_entries"][0])
        loc = int(h["namelist_location"][0])
        if loc + nbytes > self._file_size:
            raise RuntimeError(f"{self._name}: corrupt GSD file (name list past the end)")
        raw = self._pread(nbytes, loc)
        if nbytes and raw[-1] != 0:
            raise RuntimeError(f"{self._name}: corrupt GSD file (unterminated name list)")
        self._names = []
        pos = 0
        while pos < nbytes and raw[pos] != 0:
            if version < make_version(2, 0):
                name = raw[pos:pos + NAME_SIZE].split(b"\0", 1)[0]
                pos += NAME_SIZE
            else:
                end = raw.index(b"\0", pos)
                name = raw[pos:end]
                pos = end + 1
            self._names.append(name.decode())
        self._namelist_used = pos
        self._ids = {n: i for i, n in enumerate(self._names)}
        # chunk index: the used entries come first; the first zero location ends them
        cap = int(h["index_allocated_entries"][0])
        iloc = int(h["index_location"][0])
        if iloc + INDEX_DTYPE.itemsize * cap > self._file_size:
            raise RuntimeError(f"{self._name}: corrupt GSD file (index past the end)")
        index = np.frombuffer(self._pread(INDEX_DTYPE.itemsize * cap, iloc), INDEX_DTYPE)
        zero = np.flatnonzero(index["location"] == 0)
        used = int(zero[0]) if len(zero) else cap
        index = index[:used].copy()
        if used:
            sizes = (index["N"] * index["M"]).astype(np.int64) * np.array(
                [TYPE_CODES[int(t)].itemsize if int(t) in TYPE_CODES else 0
                 for t in index["type"]], np.int64)
            bad = ((~np.isin(index["type"], list(TYPE_CODES)))
                   | (index["location"] + sizes > self._file_size)
                   | (index["id"] >= len(self._names)) | (index["flags"] != 0)
                   | (np.diff(index["frame"].astype(np.int64), prepend=0) < 0))
            if bad.any():
                raise RuntimeError(f"{self._name}: corrupt GSD file (bad index entry "
                                   f"{int(np.flatnonzero(bad)[0])})")
        self._index = index
        self._lookup = {(int(f), int(i)): k for k, (f, i) in
                        enumerate(zip(index["frame"], index["id"]))}
        self._nframes = int(index["frame"][-1]) + 1 if used else 0

    # -- properties ----------------------------------------------------------------------------
    @property
    def name(self):
        return self._name

    @property
    def mode(self):
        return self._mode

    @property
    def gsd_version(self):
        return split_version(int(self._header["gsd_version"][0]))

    @property
    def schema_version(self):
        return split_version(int(self._header["schema_version"][0]))

    @property
    def schema(self):
        return self._header["schema"][0].decode()

    @property
    def application(self):
        return self._header["application"][0].decode()

    @property
    def nframes(self):
        return self._nframes

    @property
    def file_size(self):
        return self._file_size

    # -- reading -------------------------------------------------------------------------------
    def _check_open(self):
        if self._fd is None:
            raise ValueError("file is not open")

    def _entry(self, frame, name):
        i = self._ids.get(name)
        if i is None:
            return None
        k = self._lookup.get((int(frame), i))
        return None if k is None else self._index[k]

    def chunk_exists(self, frame, name):
        self._check_open()
        return self._entry(frame, name) is not None

    def read_chunk(self, frame, name):
        """The chunk's data: shape ``(N,)`` when it has one column, else ``(N, M)``."""
        self._check_open()
        if not 0 <= int(frame) < self._nframes:
            raise IndexError(f"frame {frame} is out of range (the file has {self._nframes})")
        e = self._entry(frame, name)
        if e is None:
            raise KeyError(f"{name} not found in frame {frame}")
        dt = TYPE_CODES[int(e["type"])]
        N, M = int(e["N"]), int(e["M"])
        data = np.frombuffer(self._pread(N * M * dt.itemsize, int(e["location"])), dt)
        data = data.astype(dt.newbyteorder("="), copy=True)
        return data if M == 1 else data.reshape(N, M)

    def find_matching_chunk_names(self, match):
        """Names in the file that start with ``match``."""
        self._check_open()
        return [n for n in self._names if n.startswith(match)]

    # -- writing -------------------------------------------------------------------------------
    def write_chunk(self, name, data):
        """Add a chunk to the frame being written (committed by ``end_frame``)."""
        self._check_open()
        if not self._writable:
            raise RuntimeError("file is not writable")
        name = str(name)
        if not name or len(name.encode()) >= NAME_SIZE and self.gsd_version < (2, 0):
            raise ValueError(f"invalid chunk name {name!r}")
        a = np.asarray(data)
        if a.ndim == 0:
            a = a.reshape(1)
        if a.ndim > 2:
            raise ValueError("GSD chunks are one- or two-dimensional")
        code = _type_code(a.dtype)
        a = np.ascontiguousarray(a, TYPE_CODES[code])
        if a.ndim == 2 and a.shape[1] == 0:
            raise ValueError("GSD chunks need at least one column")
        self._pending = [p for p in self._pending if p[0] != name]
        self._pending.append((name, a, code))

    def end_frame(self):
        """Commit the chunks written since the last ``end_frame`` as the next frame."""
        self._check_open()
        if not self._writable:
            raise RuntimeError("file is not writable")
        frame = self._nframes
        pending, self._pending = self._pending, []
        if not pending:
            # an empty frame counts until the file is reopened (its frame number has no entry)
            self._nframes = frame + 1
            return
        # new names get the next ids
        new_names = [n for n, _, _ in pending if n not in self._ids]
        entries = np.zeros(len(pending), INDEX_DTYPE)
        offset = self._file_size
        blobs = []
        for k, (name, a, code) in enumerate(pending):
            if name not in self._ids:
                self._ids[name] = len(self._names)
                self._names.append(name)
            N = a.shape[0]
            M = 1 if a.ndim == 1 else a.shape[1]
            entries[k] = (frame, N, offset, M, self._ids[name], code, 0)
            blobs.append(a)
            offset += a.nbytes
        # 1. the data
        pos = self._file_size
        for a in blobs:
            if a.nbytes:
                self._pwrite(a, pos)
            pos += a.nbytes
        self._file_size = pos
        # 2. new names
        if new_names:
            self._append_names(new_names)
        # 3. index entries, sorted by name id
        entries = np.sort(entries, order="id")
        self._append_index(entries)
        os.fsync(self._fd)
        self._nframes = frame + 1

    def _write_header(self):
        self._pwrite(self._header.tobytes(), 0)

    def _append_names(self, names):
        blob = b"".join(n.encode() + b"\0" for n in names)
        cap = NAME_SIZE * int(self._header["namelist_allocated_entries"][0])
        used = self._namelist_used
        if used + len(blob) <= cap:
            self._pwrite(blob, int(self._header["namelist_location"][0]) + used)
        else:
            new_cap = max(cap, NAME_SIZE)
            while new_cap < used + len(blob):
                new_cap *= 2
            old = self._pread(used, int(self._header["namelist_location"][0]))
            full = old + blob + bytes(new_cap - used - len(blob))
            loc = self._file_size
            self._pwrite(full, loc)
            self._file_size = loc + new_cap
            os.fsync(self._fd)
            self._header["namelist_location"] = loc
            self._header["namelist_allocated_entries"] = new_cap // NAME_SIZE
            self._write_header()
        self._namelist_used = used + len(blob)

    def _append_index(self, entries):
        used = len(self._index)
        cap = int(self._header["index_allocated_entries"][0])
        need = used + len(entries)
        if need > cap:
            new_cap = cap * 2
            while new_cap <= need:
                new_cap *= 2
            loc = self._file_size
            block = np.zeros(new_cap, INDEX_DTYPE)
            block[:used] = self._index
            self._pwrite(block, loc)
            self._file_size = loc + block.nbytes
            os.fsync(self._fd)
            self._header["index_location"] = loc
            self._header["index_allocated_entries"] = new_cap
            self._write_header()
        self._pwrite(entries, int(self._header["index_location"][0]) + used * INDEX_DTYPE.itemsize)
        base = used
        self._index = np.concatenate([self._index, entries])
        for k, e in enumerate(entries):
            self._lookup[(int(e["frame"]), int(e["id"]))] = base + k

    def flush(self):
        """Chunks are written at ``end_frame``; this only syncs the file."""
        self._check_open()
        if self._writable:
            os.fsync(self._fd)

    def truncate(self):
        """Remove every frame and chunk, keeping the application, schema and schema version."""
        self._check_open()
        if not self._writable:
            raise RuntimeError("file is not writable")
        h = self._header
        self._initialize(h["application"][0].decode(), h["schema"][0].decode(),
                         self.schema_version)
        self._load()
        self._pending = []

    def close(self):
        if self._fd is not None:
            os.close(self._fd)
            self._fd = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def open(name, mode="r", application=None, schema=None, schema_version=None):  # noqa: A001
    """gsd.fl.open: a ``GSDFile``."""
    return GSDFile(name, mode, application, schema, schema_version)
