"""ROOT files of flat TTrees: the on-disk layer under the step-table interchange format.

The reference reads and writes its tables through uproot (core/mu2efastsim/tables.py:25-72: `uproot.open(path)[
"dump/steps"].arrays(...)`, `uproot.recreate` + `mktree`/`extend` for TTrees), and its art dumpers write them with
ROOT's TFileService (crv/art/CrvFastSim/src/CrvStepTableDumper_module.cc:84-151: one branch per column, each a single
leaf of a basic type).  Neither uproot nor ROOT is a dependency here; this module restates the parts of ROOT's
published file format that such files use:

* file header ("root", version, fBEGIN, fEND, fSeekFree, ..., fSeekInfo, UUID; 64-bit seeks when the version is
  >= 1000000), directories (TDirectory record: dates, key-list size and seek, parent seek, UUID), key lists and keys
  (TKey: fNbytes, version (> 1000: 64-bit seeks), fObjlen, date, fKeylen, cycle, seeks, class, name, title);
* object streaming: byte counts (0x40000000), class versions, new-class tags (0xFFFFFFFF + class name) and class /
  object references (offsets into the key's buffer + 2), TObject / TNamed / TObjArray;
* TTree (class version 20), TBranch (12, 13) and its leaf (TLeafB/S/I/L/F/D/O, version 1 over TLeaf version 2); other
  branch and leaf classes (TBranchElement, TLeafElement, TLeafC, ...) are parsed far enough to be listed and skipped;
* baskets (TBasket keys) of fixed-size leaves: big-endian values, entry ranges from the branch's fBasketEntry;
* compression blocks: 9-byte header (algorithm "ZL" zlib, "XZ" LZMA, "L4" LZ4 with an XXH64 checksum, "ZS" zstd),
  compressed and uncompressed sizes (24-bit little-endian), at most 0xFFFFFF bytes per block.

Reading: RootFile(path)[ "dump/steps" ] -> Tree; Tree.arrays(columns) -> {name: native-endian array}; baskets are
decompressed on a thread pool (zlib and LZMA release the interpreter lock; LZ4 runs in the engine library's host
code).  Writing: write(path, {"dump/steps": {name: array}, ...}) makes one TTree per entry (TDirectory levels from the
path), uncompressed or zlib (ROOT's default setting 101: zlib level 1), baskets of whole clusters shared by every
branch, an empty streamer-info list (readers take the built-in layouts of these class versions), and the free-segment
record.  zstd baskets are refused with an error: no zstd decoder is available to this package.
"""
from __future__ import annotations

import ctypes
import lzma
import mmap
import os
import struct
import time as _time
import uuid
import zlib
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

BYTECOUNT = 0x40000000
NEW_CLASS = 0xFFFFFFFF
CLASS_MASK = 0x80000000
MAP_OFFSET = 2
IS_REFERENCED = 1 << 4
START_BIG_FILE = 2000000000
MAX_BLOCK = 0xFFFFFF
ROOT_VERSION = 63004            # the ROOT release number written into new files (6.30/04)
BEGIN = 100

# leaf class -> (signed dtype, unsigned dtype, branch type letter signed / unsigned)
LEAF_TYPES = {
    "TLeafB": (">i1", ">u1", "B", "b"), "TLeafS": (">i2", ">u2", "S", "s"), "TLeafI": (">i4", ">u4", "I", "i"),
    "TLeafL": (">i8", ">u8", "L", "l"), "TLeafF": (">f4", ">f4", "F", "F"), "TLeafD": (">f8", ">f8", "D", "D"),
    "TLeafO": ("?", "?", "O", "O"),
}
_DTYPE_LEAF = {np.dtype(np.int8): ("TLeafB", False), np.dtype(np.uint8): ("TLeafB", True),
               np.dtype(np.int16): ("TLeafS", False), np.dtype(np.uint16): ("TLeafS", True),
               np.dtype(np.int32): ("TLeafI", False), np.dtype(np.uint32): ("TLeafI", True),
               np.dtype(np.int64): ("TLeafL", False), np.dtype(np.uint64): ("TLeafL", True),
               np.dtype(np.float32): ("TLeafF", False), np.dtype(np.float64): ("TLeafD", False),
               np.dtype(np.bool_): ("TLeafO", False)}


class RootFormatError(ValueError):
    """The file is not a ROOT file, or uses a part of the format this reader does not cover."""


# ---------------------------------------------------------------------------------------------------------------------
# big-endian cursor

class _Cursor:
    """Big-endian reader over a buffer; `origin` is added to positions when they are used as stream tags (the offset of
    the object data inside its key's buffer, i.e. the key length)."""

    def __init__(self, buf, pos=0, origin=0):
        self.buf, self.pos, self.origin = buf, pos, origin

    def _u(self, fmt, n):
        if self.pos < 0 or self.pos + n > len(self.buf):
            raise RootFormatError("record runs past the end of its buffer")
        v = struct.unpack_from(fmt, self.buf, self.pos)[0]
        self.pos += n
        return v

    def u8(self): return self._u(">B", 1)
    def i16(self): return self._u(">h", 2)
    def u16(self): return self._u(">H", 2)
    def i32(self): return self._u(">i", 4)
    def u32(self): return self._u(">I", 4)
    def i64(self): return self._u(">q", 8)
    def f64(self): return self._u(">d", 8)

    def seek(self, big):
        return self.i64() if big else self.i32()

    def string(self):
        n = self.u8()
        if n == 255:
            n = self.i32()
        s = bytes(self.buf[self.pos:self.pos + n])
        if len(s) != n:
            raise RootFormatError("string runs past the end of its buffer")
        self.pos += n
        return s.decode("latin-1")

    def cstring(self):
        end = self.buf.find(b"\0", self.pos)
        if end < 0:
            raise RootFormatError("unterminated class name")
        s = bytes(self.buf[self.pos:end]).decode("latin-1")
        self.pos = end + 1
        return s

    def array(self, dtype, n):
        dt = np.dtype(dtype)
        if n < 0 or self.pos < 0 or self.pos + n * dt.itemsize > len(self.buf):
            raise RootFormatError("array runs past the end of its buffer")
        a = np.frombuffer(self.buf, dt, n, self.pos) if n else np.zeros(0, dt)
        self.pos += n * dt.itemsize
        return a

    def tag(self):
        return self.pos + self.origin


def _version(cur):
    """Optional byte count + class version -> (version, end position or None)."""
    start = cur.pos
    bc = cur.u32()
    if bc & BYTECOUNT and bc != NEW_CLASS:
        end = cur.pos + (bc & ~BYTECOUNT)
        return cur.i16(), end
    cur.pos = start
    return cur.i16(), None


def _skip_versioned(cur):
    _, end = _version(cur)
    if end is None:
        raise RootFormatError("expected a byte-counted record")
    cur.pos = end


def _tobject(cur):
    _version(cur)
    cur.u32()
    bits = cur.u32()
    if bits & IS_REFERENCED:
        cur.u16()


def _tnamed(cur):
    _, end = _version(cur)
    _tobject(cur)
    name, title = cur.string(), cur.string()
    if end is not None:
        cur.pos = end
    return name, title


@dataclass
class _Ctx:
    classes: dict = field(default_factory=dict)     # tag -> class name
    objects: dict = field(default_factory=dict)     # tag -> object


def _object_any(cur, ctx):
    """A pointer member / collection element: null, a reference to an object already read, or a (new or referenced)
    class followed by the object."""
    start = cur.pos
    bc = cur.u32()
    if bc == 0:
        return None
    if not (bc & BYTECOUNT) or bc == NEW_CLASS:
        if bc != NEW_CLASS:
            return ctx.objects.get(bc)                 # object reference
        end, tagpos, tag = None, start, bc             # new class without a byte count (old writers)
    else:
        end = cur.pos + (bc & ~BYTECOUNT)
        tagpos = cur.pos
        tag = cur.u32()
    if tag == NEW_CLASS:
        cname = cur.cstring()
        ctx.classes[tagpos + cur.origin + MAP_OFFSET] = cname
    elif tag & CLASS_MASK:
        cname = ctx.classes.get(tag & ~CLASS_MASK)
        if cname is None:
            raise RootFormatError("reference to a class that was not defined earlier in the record")
    else:
        raise RootFormatError("malformed object header")
    obj = _read_class(cname, cur, ctx)
    ctx.objects[start + cur.origin + MAP_OFFSET] = obj
    if end is not None:
        cur.pos = end
    return obj


def _objarray(cur, ctx):
    _, end = _version(cur)
    _tobject(cur)
    cur.string()
    n = cur.i32()
    cur.i32()
    items = [_object_any(cur, ctx) for _ in range(n)]
    if end is not None:
        cur.pos = end
    return items


# ---------------------------------------------------------------------------------------------------------------------
# TTree / TBranch / TLeaf

@dataclass
class Leaf:
    cls: str
    name: str
    title: str
    length: int
    size: int
    unsigned: bool
    leaf_count: object = None                    # the counter leaf of a counted array (name[nname])

    def dtype(self):
        t = LEAF_TYPES.get(self.cls)
        if t is None:
            return None
        return np.dtype(t[1] if self.unsigned else t[0])


@dataclass
class Branch:
    cls: str
    name: str
    title: str
    entries: int
    write_basket: int
    basket_bytes: np.ndarray
    basket_entry: np.ndarray
    basket_seek: np.ndarray
    leaves: list
    branches: list
    embedded_baskets: int
    entry_offset_len: int = 0
    class_name: str = ""                         # TBranchElement: the streamed class (e.g. vector<short>)


class _Unsupported:
    def __init__(self, cls):
        self.cls = cls


def _leaf(cls, cur, ctx):
    _, end = _version(cur)
    _, lend = _version(cur)                      # TLeaf base
    name, title = _tnamed(cur)
    length, size, _off = cur.i32(), cur.i32(), cur.i32()
    cur.u8()
    unsigned = bool(cur.u8())
    count = _object_any(cur, ctx)                # fLeafCount
    if lend is not None:
        cur.pos = lend
    if end is not None:
        cur.pos = end
    return Leaf(cls, name, title, length, size, unsigned, count if isinstance(count, Leaf) else None)


def _branch(cls, cur, ctx):
    v, end = _version(cur)
    if cls != "TBranch":
        b = _branch("TBranch", cur, ctx)         # base part of a derived branch class
        b.cls = cls
        if cls == "TBranchElement":
            try:
                b.class_name = cur.string()      # fClassName, the first member after the base
            except RootFormatError:
                b.class_name = ""
        if end is not None:
            cur.pos = end
        return b
    if v not in (12, 13):
        raise RootFormatError(f"TBranch class version {v}: versions 12 and 13 are read")
    name, title = _tnamed(cur)
    _skip_versioned(cur)                         # TAttFill
    cur.i32(), cur.i32()                         # fCompress, fBasketSize
    entry_offset_len = cur.i32()
    write_basket = cur.i32()
    cur.i64()                                    # fEntryNumber
    if v >= 13:
        _skip_versioned(cur)                     # fIOFeatures
    cur.i32()                                    # fOffset
    max_baskets = cur.i32()
    cur.i32()                                    # fSplitLevel
    entries = cur.i64()
    cur.i64(), cur.i64(), cur.i64()              # fFirstEntry, fTotBytes, fZipBytes
    branches = _objarray(cur, ctx)
    leaves = _objarray(cur, ctx)
    baskets = _objarray(cur, ctx)
    arrs = []
    for dt in (">i4", ">i8", ">i8"):
        arrs.append(cur.array(dt, max_baskets) if cur.u8() else np.zeros(max_baskets, dt))
    cur.string()                                 # fFileName
    if end is not None:
        cur.pos = end
    emb = sum(1 for b in baskets if b is not None)
    return Branch(cls, name, title, entries, write_basket, arrs[0].astype(np.int64), arrs[1].astype(np.int64),
                  arrs[2].astype(np.int64), [x for x in leaves if x is not None],
                  [x for x in branches if x is not None], emb, entry_offset_len)


def _read_class(cname, cur, ctx):
    if cname.startswith("TBranch"):
        return _branch(cname, cur, ctx)
    if cname.startswith("TLeaf"):
        return _leaf(cname, cur, ctx)
    return _Unsupported(cname)                   # skipped through its byte count by the caller


def _ttree(cur, ctx):
    v, end = _version(cur)
    if v != 20:
        raise RootFormatError(f"TTree class version {v}: version 20 (ROOT 6) is read")
    name, title = _tnamed(cur)
    for _ in range(3):                           # TAttLine, TAttFill, TAttMarker
        _skip_versioned(cur)
    entries = cur.i64()
    for _ in range(4):                           # fTotBytes, fZipBytes, fSavedBytes, fFlushedBytes
        cur.i64()
    cur.f64()                                    # fWeight
    cur.i32(), cur.i32(), cur.i32(), cur.i32()   # fTimerInterval, fScanField, fUpdate, fDefaultEntryOffsetLen
    nclus = cur.i32()
    for _ in range(6):                           # fMaxEntries .. fEstimate
        cur.i64()
    for _ in range(2):                           # fClusterRangeEnd, fClusterSize
        if cur.u8():
            cur.array(">i8", nclus)
    _skip_versioned(cur)                         # fIOFeatures
    branches = [b for b in _objarray(cur, ctx) if b is not None]
    leaves = None
    try:                                         # the rest: the tree's leaf list (references into the branches) ..
        leaves = _objarray(cur, ctx)
        _object_any(cur, ctx)                    # fAliases
        cur.array(">f8", cur.i32())              # fIndexValues
        cur.array(">i4", cur.i32())              # fIndex
        for _ in range(4):                       # fTreeIndex, fFriends, fUserInfo, fBranchRef
            _object_any(cur, ctx)
        if end is not None and cur.pos != end:
            leaves = None
    except (RootFormatError, struct.error):      # .. is not needed to read columns
        leaves = None
    return name, title, entries, branches, leaves


# ---------------------------------------------------------------------------------------------------------------------
# compression

def _native():
    from . import _capi
    return _capi.load()


def _lz4(block, usize):
    if len(block) < 8:
        raise RootFormatError("LZ4 block shorter than its checksum")
    L = _native()
    src = bytes(block[8:])
    want = int.from_bytes(bytes(block[:8]), "big")
    if L.crv_xxh64(src, len(src), 0) != want:
        raise RootFormatError("LZ4 block checksum mismatch")
    out = ctypes.create_string_buffer(usize)
    n = L.crv_lz4_block_decompress(src, len(src), out, usize)
    if n != usize:
        raise RootFormatError("LZ4 block does not decompress to its stated size")
    return out.raw


def decompress(buf, objlen):
    """Concatenated ROOT compression blocks -> `objlen` bytes."""
    out, pos = [], 0
    got = 0
    while got < objlen:
        h = bytes(buf[pos:pos + 9])
        if len(h) < 9:
            raise RootFormatError("compressed object ends inside a block header")
        alg = h[:2]
        csize = h[3] | (h[4] << 8) | (h[5] << 16)
        usize = h[6] | (h[7] << 8) | (h[8] << 16)
        block = buf[pos + 9:pos + 9 + csize]
        if len(block) != csize:
            raise RootFormatError("compressed block runs past the end of its key")
        if alg == b"ZL":
            try:
                data = zlib.decompress(block)
            except zlib.error as exc:
                raise RootFormatError(f"corrupt zlib block: {exc}") from None
        elif alg == b"XZ":
            try:
                data = lzma.decompress(block)
            except lzma.LZMAError as exc:
                raise RootFormatError(f"corrupt LZMA block: {exc}") from None
        elif alg == b"L4":
            data = _lz4(block, usize)
        elif alg == b"ZS":
            raise RootFormatError("zstd-compressed objects: no zstd decoder is available here")
        else:
            raise RootFormatError(f"compression algorithm {alg!r} is not read")
        if len(data) != usize:
            raise RootFormatError("block does not decompress to its stated size")
        out.append(data)
        got += usize
        pos += 9 + csize
    return b"".join(out)


def _block(alg, method, chunk, body):
    return alg + bytes([method]) + len(body).to_bytes(3, "little") + len(chunk).to_bytes(3, "little") + body


def compress(raw, setting=101):
    """ROOT compression blocks of `raw` (each at most 0xFFFFFF input bytes) for a ROOT compression setting
    (algorithm x 100 + level: 1xx zlib, 2xx LZMA; 1..9 alone mean zlib); None when it does not shrink the data."""
    alg, level = divmod(int(setting), 100) if setting >= 100 else (1, int(setting))
    out = []
    for a in range(0, len(raw), MAX_BLOCK):
        chunk = raw[a:a + MAX_BLOCK]
        if alg == 1:
            out.append(_block(b"ZL", 8, chunk, zlib.compress(chunk, level)))
        elif alg == 2:
            out.append(_block(b"XZ", 0, chunk, lzma.compress(chunk, preset=level)))
        else:
            raise ValueError(f"compression setting {setting}: zlib (1xx) and LZMA (2xx) are written")
    z = b"".join(out)
    return z if len(z) < len(raw) else None


# ---------------------------------------------------------------------------------------------------------------------
# reading

@dataclass
class Key:
    nbytes: int
    version: int
    objlen: int
    datime: int
    keylen: int
    cycle: int
    seek_key: int
    seek_pdir: int
    classname: str
    name: str
    title: str


def _key(cur):
    nbytes, version, objlen, datime = cur.i32(), cur.i16(), cur.i32(), cur.u32()
    keylen, cycle = cur.i16(), cur.i16()
    big = version > 1000
    seek_key, seek_pdir = cur.seek(big), cur.seek(big)
    return Key(nbytes, version, objlen, datime, keylen, cycle, seek_key, seek_pdir & 0xFFFFFFFFFFFF, cur.string(),
               cur.string(), cur.string())


_VECTOR = {f"vector<{k}>": v for k, v in (
    ("char", ">i1"), ("unsignedchar", ">u1"), ("short", ">i2"), ("unsignedshort", ">u2"), ("int", ">i4"),
    ("unsignedint", ">u4"), ("long", ">i8"), ("longlong", ">i8"), ("Long64_t", ">i8"), ("unsignedlong", ">u8"),
    ("unsignedlonglong", ">u8"), ("ULong64_t", ">u8"), ("float", ">f4"), ("double", ">f8"), ("bool", "?"),
    ("Short_t", ">i2"), ("Int_t", ">i4"), ("Float_t", ">f4"), ("Double_t", ">f8"))}


_VECTOR_OF = {">i1": "vector<char>", ">u1": "vector<unsigned char>", ">i2": "vector<short>",
              ">u2": "vector<unsigned short>", ">i4": "vector<int>", ">u4": "vector<unsigned int>",
              ">i8": "vector<long>",
              ">u8": "vector<unsigned long>", ">f4": "vector<float>", ">f8": "vector<double>", "|b1": "vector<bool>"}


class JaggedArray:
    """Variable-length rows: values (flat) and offsets (rows + 1); row i is values[offsets[i]:offsets[i + 1]]."""

    def __init__(self, values, offsets):
        self.values = np.asarray(values)
        self.offsets = np.asarray(offsets, np.int64)
        if self.offsets.ndim != 1 or len(self.offsets) < 1 or self.offsets[0] != 0 or \
                self.offsets[-1] != len(self.values) or np.any(np.diff(self.offsets) < 0):
            raise ValueError("offsets must start at 0, not decrease, and end at the number of values")

    @classmethod
    def from_rows(cls, rows, dtype=None):
        rows = [np.asarray(r, dtype) for r in rows]
        cnt = np.array([len(r) for r in rows], np.int64)
        dt = dtype or (rows[0].dtype if rows else np.float64)
        vals = np.concatenate(rows).astype(dt) if rows else np.zeros(0, dt)
        return cls(vals, np.r_[0, np.cumsum(cnt)])

    @property
    def counts(self):
        return np.diff(self.offsets)

    @property
    def nbytes(self):
        return self.values.nbytes + self.offsets.nbytes

    @property
    def dtype(self):
        return self.values.dtype

    def __len__(self):
        return len(self.offsets) - 1

    def __getitem__(self, i):
        return self.values[self.offsets[i]:self.offsets[i + 1]]

    def tolist(self):
        return [self[i].tolist() for i in range(len(self))]

    def __eq__(self, other):
        return isinstance(other, JaggedArray) and np.array_equal(self.offsets, other.offsets) and \
            self.values.dtype == other.values.dtype and np.array_equal(self.values, other.values)

    __hash__ = None

    def take(self, sel):
        sel = np.arange(len(self))[sel]
        return JaggedArray.from_rows([self[i] for i in sel], self.values.dtype)


class Tree:
    """One TTree: name, title, entries and branches {name: Branch}; arrays() reads fixed-size leaf columns."""

    def __init__(self, file, key):
        self.file, self.key = file, key
        buf = file.object_bytes(key)
        cur = _Cursor(buf, 0, key.keylen)
        self.name, self.title, self.num_entries, branches, self.leaves = _ttree(cur, _Ctx())
        self.branches = {b.name: b for b in branches}

    def __len__(self):
        return self.num_entries

    def keys(self):
        return list(self.branches)

    def _layout(self, b):
        """(dtype, values per entry, jagged header bytes or None): fixed leaves, counted arrays (header 0) and
        std::vector<basic> element branches (10 header bytes per entry: byte count, version, size)."""
        if b.cls == "TBranchElement" and not b.branches:
            m = _VECTOR.get(b.class_name.replace(" ", ""))
            if m is None:
                raise RootFormatError(f"branch {b.name!r}: class {b.class_name!r} is not a vector of a basic type")
            return np.dtype(m), 1, 10
        if b.branches or len(b.leaves) != 1 or not isinstance(b.leaves[0], Leaf) or b.leaves[0].dtype() is None:
            raise RootFormatError(f"branch {b.name!r} ({b.cls}) is not a single leaf of a basic type")
        lf = b.leaves[0]
        if lf.leaf_count is not None:
            return lf.dtype(), max(1, lf.length), 0
        return lf.dtype(), max(1, lf.length), None

    def _column(self, b):
        dt, per, header = self._layout(b)
        if not (0 <= b.write_basket < len(b.basket_entry)) or b.entries < 0:
            raise RootFormatError(f"branch {b.name!r}: basket count outside its tables")
        if int(b.basket_entry[b.write_basket]) < b.entries or b.embedded_baskets:
            raise RootFormatError(f"branch {b.name!r}: entries held in an unflushed (embedded) basket are not read")
        be = b.basket_entry[:b.write_basket + 1]
        if be[0] != 0 or np.any(np.diff(be) < 0) or int(be[-1]) != b.entries:
            raise RootFormatError(f"branch {b.name!r}: basket entry ranges do not cover its entries")
        jobs = []
        for i in range(b.write_basket):
            a, e = int(b.basket_entry[i]), int(b.basket_entry[i + 1])
            if e > a:
                jobs.append((int(b.basket_seek[i]), int(b.basket_bytes[i]), a, e))

        def basket(job):
            seek, nbytes, a, e = job
            kc = _Cursor(self.file.buf, seek)
            k = _key(kc)
            if k.nbytes != nbytes:
                raise RootFormatError(f"branch {b.name!r}: basket at {seek} does not match the branch's byte count")
            kc.i16()
            bufsize = kc.i32()
            if bufsize < 0:                      # extra IO-bits byte
                kc.u8()
            kc.i32(), kc.i32()                   # fNevBufSize, fNevBuf
            last = kc.i32()
            return k, last, self.file.object_bytes(k)

        if header is None:
            out = np.empty(b.entries * per, dt.newbyteorder("="))

            def fixed(job):
                k, _, raw = basket(job)
                a, e = job[2], job[3]
                n = (e - a) * per
                if len(raw) < n * dt.itemsize:
                    raise RootFormatError(f"branch {b.name!r}: basket at {job[0]} holds fewer values than its entries")
                out[a * per:e * per] = np.frombuffer(raw, dt, n)
            self._map(fixed, jobs)
            return out.reshape(-1, per) if per > 1 else out
        parts = [None] * len(jobs)

        def jag(ij):
            i, job = ij
            k, last, raw = basket(job)
            a, e = job[2], job[3]
            border = last - k.keylen
            if border < 0 or border + 4 * (e - a + 2) > len(raw):
                raise RootFormatError(f"branch {b.name!r}: basket at {job[0]} has no entry offsets")
            offs = np.frombuffer(raw, ">i4", e - a + 1, border + 4).astype(np.int64) - k.keylen
            offs[-1] = border
            starts, ends = offs[:-1] + header, offs[1:]
            if np.any(ends < starts) or np.any((ends - starts) % dt.itemsize):
                raise RootFormatError(f"branch {b.name!r}: basket at {job[0]} has inconsistent entry offsets")
            cnt = (ends - starts) // dt.itemsize
            body = np.frombuffer(raw, np.uint8, border)
            idx = np.repeat(starts - np.r_[0, np.cumsum((ends - starts))[:-1]], ends - starts) + \
                np.arange(int((ends - starts).sum()))
            parts[i] = (cnt, body[idx].view(dt) if len(idx) else np.zeros(0, dt))
        self._map(jag, list(enumerate(jobs)))
        counts = np.concatenate([p[0] for p in parts]) if parts else np.zeros(0, np.int64)
        values = np.concatenate([p[1] for p in parts]).astype(dt.newbyteorder("=")) if parts else \
            np.zeros(0, dt.newbyteorder("="))
        return JaggedArray(values, np.r_[0, np.cumsum(counts)].astype(np.int64))

    def _map(self, fn, jobs):
        if len(jobs) > 1 and self.file.threads > 1:
            with ThreadPoolExecutor(self.file.threads) as ex:
                list(ex.map(fn, jobs))
        else:
            for j in jobs:
                fn(j)

    def arrays(self, columns=None):
        """{column: native-endian array} for `columns` (all when None), in branch order."""
        names = list(self.branches) if columns is None else list(columns)
        missing = [c for c in names if c not in self.branches]
        if missing:
            raise KeyError(f"tree {self.name!r} has no branches {missing}")
        return {c: self._column(self.branches[c]) for c in names}


class RootFile:
    """A ROOT file opened read-only (memory-mapped).  f["dump/steps"] -> Tree; f.keys() lists the paths."""

    def __init__(self, path, threads=None):
        self.path = path
        self._fh = open(path, "rb")
        size = os.fstat(self._fh.fileno()).st_size
        if size < 64:
            self._fh.close()
            raise RootFormatError(f"{path}: not a ROOT file (too short)")
        self.buf = mmap.mmap(self._fh.fileno(), 0, access=mmap.ACCESS_READ)
        self.threads = threads or min(16, os.cpu_count() or 1)
        cur = _Cursor(self.buf)
        if bytes(self.buf[:4]) != b"root":
            self.close()
            raise RootFormatError(f"{path}: not a ROOT file (no 'root' magic)")
        cur.pos = 4
        self.version = cur.i32()
        big = self.version >= 1000000
        self.begin = cur.i32()
        self.end, self.seek_free = cur.seek(big), cur.seek(big)
        self.nbytes_free, self.nfree, self.nbytes_name = cur.i32(), cur.i32(), cur.i32()
        self.units, self.compression = cur.u8(), cur.i32()
        self.seek_info, self.nbytes_info = cur.seek(big), cur.i32()
        self.top = self._directory(self.begin + self.nbytes_name)

    def close(self):
        try:
            self.buf.close()
        finally:
            self._fh.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _directory(self, pos):
        cur = _Cursor(self.buf, pos)
        v = cur.i16()
        cur.u32(), cur.u32()
        nbytes_keys, _ = cur.i32(), cur.i32()
        big = v > 1000
        cur.seek(big), cur.seek(big)
        seek_keys = cur.seek(big)
        keys = []
        if seek_keys:
            kc = _Cursor(self.buf, seek_keys)
            _key(kc)
            for _ in range(kc.i32()):
                keys.append(_key(kc))
        return keys

    def object_bytes(self, key):
        a = key.seek_key + key.keylen
        data = self.buf[a:key.seek_key + key.nbytes]
        if key.objlen == key.nbytes - key.keylen:
            return data
        return decompress(data, key.objlen)

    def _lookup(self, keys, name):
        cyc = None
        if ";" in name:
            name, c = name.split(";", 1)
            cyc = int(c)
        hits = [k for k in keys if k.name == name and (cyc is None or k.cycle == cyc)]
        if not hits:
            raise KeyError(name)
        return max(hits, key=lambda k: k.cycle)

    def get_key(self, path):
        keys = self.top
        parts = [p for p in path.split("/") if p]
        for i, p in enumerate(parts):
            k = self._lookup(keys, p)
            if i == len(parts) - 1:
                return k
            if k.classname not in ("TDirectory", "TDirectoryFile"):
                raise KeyError(f"{p} is a {k.classname}, not a directory")
            keys = self._directory(k.seek_key + k.keylen)
        raise KeyError(path)

    def __getitem__(self, path):
        k = self.get_key(path)
        if k.classname != "TTree":
            raise RootFormatError(f"{path} is a {k.classname}; TTrees are read")
        return Tree(self, k)

    def keys(self, keys=None, prefix=""):
        """Every object path, directories first-level order."""
        out = []
        for k in (self.top if keys is None else keys):
            p = f"{prefix}{k.name}"
            out.append(p)
            if k.classname in ("TDirectory", "TDirectoryFile"):
                out += self.keys(self._directory(k.seek_key + k.keylen), p + "/")
        return out


# ---------------------------------------------------------------------------------------------------------------------
# writing

class _W:
    """Big-endian record builder; positions used as stream tags include `origin` (the key length)."""

    def __init__(self, origin=0):
        self.b = bytearray()
        self.origin = origin
        self.classes = {}

    def put(self, fmt, *v):
        self.b += struct.pack(fmt, *v)

    def string(self, s):
        s = s.encode("latin-1")
        if len(s) < 255:
            self.b.append(len(s))
        else:
            self.b.append(255)
            self.put(">i", len(s))
        self.b += s

    def begin(self, version):
        at = len(self.b)
        self.put(">Ih", 0, version)
        return at

    def end(self, at):
        struct.pack_into(">I", self.b, at, (len(self.b) - at - 4) | BYTECOUNT)

    def tobject(self):
        self.put(">hII", 1, 0, 0)

    def tnamed(self, name, title):
        at = self.begin(1)
        self.tobject()
        self.string(name)
        self.string(title)
        self.end(at)

    def versioned(self, version, fmt, *v):
        at = self.begin(version)
        self.put(fmt, *v)
        self.end(at)

    def object_any(self, cname, body):
        """Write an object behind its class tag; returns the object's tag for later references."""
        cnt = len(self.b)
        self.put(">I", 0)
        if cname in self.classes:
            self.put(">I", self.classes[cname] | CLASS_MASK)
        else:
            self.classes[cname] = len(self.b) + self.origin + MAP_OFFSET
            self.put(">I", NEW_CLASS)
            self.b += cname.encode("latin-1") + b"\0"
        tag = cnt + self.origin + MAP_OFFSET
        body(self)
        struct.pack_into(">I", self.b, cnt, (len(self.b) - cnt - 4) | BYTECOUNT)
        return tag

    def objarray(self, items):
        """items: list of (class name, body) or ("ref", tag)."""
        at = self.begin(3)
        self.tobject()
        self.string("")
        self.put(">ii", len(items), 0)
        for cname, x in items:
            if cname == "ref":
                self.put(">I", x)
            else:
                self.object_any(cname, x)
        self.end(at)


def _datime(t=None):
    t = _time.localtime(t)
    return ((t.tm_year - 1995) << 26) | (t.tm_mon << 22) | (t.tm_mday << 17) | (t.tm_hour << 12) | (t.tm_min << 6) | \
        t.tm_sec


def _tstring_len(s):
    n = len(s.encode("latin-1"))
    return n + (1 if n < 255 else 5)


def _keylen(big, cname, name, title):
    return 26 + (8 if big else 0) + _tstring_len(cname) + _tstring_len(name) + _tstring_len(title)


def _key_header(big, nbytes, objlen, keylen, cycle, seek_key, seek_pdir, cname, name, title, datime):
    w = _W()
    w.put(">ihiIhh", nbytes, 1004 if big else 4, objlen, datime, keylen, cycle)
    w.put(">qq" if big else ">ii", seek_key, seek_pdir)
    for s in (cname, name, title):
        w.string(s)
    assert len(w.b) == _keylen(big, cname, name, title)
    return bytes(w.b)


def _dir_record(big, datime, nbytes_keys, nbytes_name, seek_dir, seek_parent, seek_keys, uid):
    w = _W()
    w.put(">hIIii", 1005 if big else 5, datime, datime, nbytes_keys, nbytes_name)
    if big:
        w.put(">qqq", seek_dir, seek_parent, seek_keys)
    else:
        w.put(">iii", seek_dir, seek_parent, seek_keys)
    w.put(">h", 1)
    w.b += uid
    if not big:
        w.put(">iii", 0, 0, 0)
    assert len(w.b) == 60
    return bytes(w.b)


@dataclass
class _Col:
    name: str
    data: object             # (entries,) or (entries, n) native array, or a JaggedArray
    leaf: str
    unsigned: bool
    per: int
    counter: str = ""        # counted array: the name of its counter column
    vector: str = ""         # std::vector element branch (tests): the vector's class name

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def variable(self):
        return bool(self.counter or self.vector)

    def raw(self, a, e, be, keylen):
        """Big-endian bytes of entries [a, e) (variable-size rows: values, then the entry-offset block; a
        std::vector row is preceded by its byte count, version and size)."""
        if not self.variable:
            return np.ascontiguousarray(self.data[a:e]).astype(be, copy=False).tobytes()
        o = self.data.offsets
        if self.vector:
            rows = []
            for i in range(a, e):
                v = self.data.values[o[i]:o[i + 1]].astype(be, copy=False).tobytes()
                rows.append(struct.pack(">Ihi", (6 + len(v)) | BYTECOUNT, 9, o[i + 1] - o[i]) + v)
            starts = np.r_[0, np.cumsum([len(r) for r in rows])[:-1]].astype(np.int64) + keylen if rows else \
                np.zeros(0, np.int64)
            vals = b"".join(rows)
        else:
            vals = self.data.values[o[a]:o[e]].astype(be, copy=False).tobytes()
            starts = (o[a:e] - o[a]) * be.itemsize + keylen
        offs = np.r_[e - a + 1, starts, 0].astype(">i4")
        return vals + offs.tobytes()


ENTRY_OFFSET_LEN = 1000          # ROOT's default entry-offset table length for variable-size branches


def _columns(cols, vectors=()):
    out = []
    n = None
    names = set(cols)
    for name, a in cols.items():
        if not isinstance(a, JaggedArray) and isinstance(a, (list, tuple)) and a and \
                not np.isscalar(a[0]) and np.ndim(a[0]) == 1:
            a = JaggedArray.from_rows(a)
        jag = isinstance(a, JaggedArray)
        if not jag:
            a = np.asarray(a)
        if a.dtype not in _DTYPE_LEAF:
            raise TypeError(f"column {name!r}: dtype {a.dtype} has no ROOT leaf type (basic numeric types only)")
        if not jag and a.ndim not in (1, 2):
            raise ValueError(f"column {name!r}: one value, a fixed-length array or a variable-length row per entry")
        if n is None:
            n = len(a)
        elif len(a) != n:
            raise ValueError("every column of a tree needs the same number of entries")
        leaf, uns = _DTYPE_LEAF[a.dtype]
        if jag and name in vectors:
            out.append(_Col(name, a, leaf, uns, 1, "", _VECTOR_OF[np.dtype(LEAF_TYPES[leaf][1 if uns else 0]).str]))
        elif jag:
            cname = f"n{name}"
            cnt = a.counts.astype(np.int32)
            if cname in names:
                given = [c for c in out if c.name == cname]
                if not given or not np.array_equal(given[0].data, cnt):
                    raise ValueError(f"column {cname!r} must come before {name!r} and hold its row lengths")
            else:
                out.append(_Col(cname, cnt, "TLeafI", False, 1))
            out.append(_Col(name, a, leaf, uns, 1, cname))
        else:
            out.append(_Col(name, a, leaf, uns, 1 if a.ndim == 1 else a.shape[1]))
    return out, (n or 0)


def _leaf_body(c, lo, hi, leaf_tags):
    t = LEAF_TYPES[c.leaf]
    dt = np.dtype(t[1] if c.unsigned else t[0])
    size = dt.itemsize

    def body(w):
        if c.vector:                                   # TLeafElement: TLeaf, fID, fType
            at = w.begin(1)
            lat = w.begin(2)
            w.tnamed(c.name, c.name)
            w.put(">iiiBB", 0, size, 0, 0, 0)
            w.put(">I", 0)
            w.end(lat)
            w.put(">ii", -1, 0)
            w.end(at)
            return
        at = w.begin(1)
        lat = w.begin(2)
        w.tnamed(c.name, f"{c.name}[{c.counter}]" if c.counter else c.name)
        w.put(">iiiBB", c.per, size, 0, 0, 1 if c.unsigned else 0)
        w.put(">I", leaf_tags[c.counter] if c.counter else 0)   # fLeafCount: a reference to the counter's leaf
        w.end(lat)
        w.b += np.array([lo, hi], dt).tobytes()
        w.end(at)
    return body


def _branch_body(c, lo, hi, nbk, n, bounds, seeks, nbytes, tot, zip_, fcompress, leaf_tags):
    letter = LEAF_TYPES[c.leaf][3 if c.unsigned else 2]
    if c.vector:
        btitle = c.name
    elif c.counter:
        btitle = f"{c.name}[{c.counter}]/{letter}"
    else:
        btitle = f"{c.name}[{c.per}]/{letter}" if c.per > 1 else f"{c.name}/{letter}"
    mb = max(10, nbk + 1)

    def body(w):
        if c.vector:                                   # TBranchElement: the TBranch base, then its own members
            ea = w.begin(10)
            base(w)
            for x in (c.vector, "", ""):               # fClassName, fParentName, fClonesName
                w.string(x)
            w.put(">Ihiiii", 0, 6, -1, 0, -1, 0)       # fCheckSum, fClassVersion, fID, fType, fStreamerType, ..
            w.put(">II", 0, 0)                         # fBranchCount, fBranchCount2
            w.end(ea)
        else:
            base(w)

    def base(w):
        at = w.begin(13)
        w.tnamed(c.name, btitle)
        w.versioned(2, ">hh", 0, 1001)                 # TAttFill
        w.put(">iiiiq", fcompress, 32000, ENTRY_OFFSET_LEN if c.variable else 0, nbk, n)
        w.versioned(1, ">B", 0)                        # fIOFeatures
        w.put(">iii", 0, mb, 0)                        # fOffset, fMaxBaskets, fSplitLevel
        w.put(">qqqq", n, 0, tot, zip_)                # fEntries, fFirstEntry, fTotBytes, fZipBytes
        w.objarray([])                                 # fBranches
        la = w.begin(3)                                # fLeaves: the one leaf, kept for the tree's references
        w.tobject()
        w.string("")
        w.put(">ii", 1, 0)
        leaf_tags[c.name] = w.object_any("TLeafElement" if c.vector else c.leaf, _leaf_body(c, lo, hi, leaf_tags))
        w.end(la)
        w.objarray([])                                 # fBaskets: every basket is a key of its own
        bb, be, bs = np.zeros(mb, ">i4"), np.zeros(mb, ">i8"), np.zeros(mb, ">i8")
        bb[:nbk], be[:nbk + 1], bs[:nbk] = nbytes, bounds, seeks
        for arr in (bb, be, bs):
            w.put(">B", 1)
            w.b += arr.tobytes()
        w.string("")                                   # fFileName
        w.end(at)
    return body


def write(path, trees, compression=101, basket_bytes=4 << 20, title="", threads=None, _compressor=None, _vectors=()):
    """Write {"dir/.../tree": {column: array}} as TTrees (directories made from the path).  compression: ROOT
    setting (0 none, 1xx zlib level xx (the default 101 is ROOT's), 2xx LZMA; 1..9 alone mean zlib).  Every branch of
    a tree shares the basket (cluster) boundaries; a basket holds about `basket_bytes` of the tree's widest column.
    Empty or None tables are skipped, as in the reference's write.  Variable-length columns (JaggedArray, or a list
    of 1-d arrays) are written as counted arrays with a counter column n<name>, as uproot writes them.  Tests only:
    _compressor (raw bytes -> blocks or None, instead of the setting's algorithm) and _vectors (names of variable
    columns to write as std::vector element branches, the layout ROOT's TTree::Branch gives a vector of a basic type,
    which this module reads from files ROOT made; these records are not checked against ROOT here)."""
    threads = threads or min(16, os.cpu_count() or 1)
    items = []
    for tpath, cols in trees.items():
        if cols is None:
            continue
        cc, n = _columns(cols, _vectors)
        if n == 0 or not cc:
            continue
        parts = [p for p in tpath.split("/") if p]
        if not parts:
            raise ValueError("empty tree path")
        items.append((tuple(parts[:-1]), parts[-1], cc, n))
    est = sum(c.data.nbytes + 4096 for _, _, cc, _ in items for c in cc) + (1 << 20)
    big = est > START_BIG_FILE - (64 << 20)
    fname = os.path.basename(path)
    now = _datime()
    uid = uuid.uuid4().bytes
    comp = int(compression or 0)
    fcompress = comp if comp >= 100 else (100 + comp if comp else 0)
    pack = _compressor or (lambda r: compress(r, fcompress))
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    dirs = {}                                          # directory path -> {pos, keylen, keys, hdr, seek_keys, ...}
    for dparts, _, _, _ in items:
        for i in range(1, len(dparts) + 1):
            dirs.setdefault(dparts[:i], {})
    with open(path, "wb") as f:
        pos = 0

        def emit(b):
            nonlocal pos
            f.write(b)
            pos += len(b)

        emit(b"\0" * BEGIN)
        top_keylen = _keylen(big, "TFile", fname, title)
        namelen = _tstring_len(fname) + _tstring_len(title)
        top_nbytes = top_keylen + namelen + 60
        emit(b"\0" * top_nbytes)                      # top directory: filled in at the end
        for d, rec in dirs.items():
            rec.update(pos=pos, keylen=_keylen(big, "TDirectory", d[-1], ""), keys=[])
            emit(b"\0" * (rec["keylen"] + 60))
        top_keys = []

        def seek_dir(d):
            return dirs[d]["pos"] if d else BEGIN

        def write_key(cname, name, ttl, raw, pdir, compress_it=True):
            z = pack(raw) if (comp and compress_it and len(raw) > 256) else None
            payload = z if z is not None else raw
            kl = _keylen(big, cname, name, ttl)
            at = pos
            hdr = _key_header(big, kl + len(payload), len(raw), kl, 1, at, pdir, cname, name, ttl, now)
            emit(hdr + payload)
            return at, kl + len(payload), hdr

        for d, tname, cc, n in items:
            pdir = seek_dir(d)
            def entry_bytes(c):
                if c.variable:
                    return c.dtype.itemsize * max(1, -(-len(c.data.values) // max(1, n))) + 4 + (10 if c.vector else 0)
                return c.dtype.itemsize * c.per
            per_basket = max(1, min(n, basket_bytes // max(entry_bytes(c) for c in cc)))
            bounds = list(range(0, n, per_basket)) + [n]
            nbk = len(bounds) - 1
            info = []
            for c in cc:
                t = LEAF_TYPES[c.leaf]
                be = np.dtype(t[1] if c.unsigned else t[0])
                kl = _keylen(big, "TBasket", c.name, tname) + 19
                raws = [c.raw(bounds[i], bounds[i + 1], be, kl) for i in range(nbk)]
                zs = [None] * nbk
                if comp:
                    with ThreadPoolExecutor(threads) as ex:
                        zs = list(ex.map(lambda r: pack(r) if len(r) > 256 else None, raws))
                seeks, nbytes, tot, zip_ = [], [], 0, 0
                for i in range(nbk):
                    raw = raws[i]
                    payload = zs[i] if zs[i] is not None else raw
                    nb = kl + len(payload)
                    ne = bounds[i + 1] - bounds[i]
                    data_len = len(raw) - (4 * (ne + 2) if c.variable else 0)
                    hdr = _key_header(big, nb, len(raw), kl, 1, pos, pdir, "TBasket", c.name, tname, now)
                    # TBasket header: version, fBufferSize, fNevBufSize, fNevBuf, fLast, flag
                    nevbufsize = ENTRY_OFFSET_LEN if c.variable else be.itemsize * c.per
                    bh = struct.pack(">hiiiiB", 3, kl + len(raw), nevbufsize, ne, kl + data_len, 0)
                    seeks.append(pos)
                    nbytes.append(nb)
                    tot += kl + len(raw)
                    zip_ += nb
                    emit(hdr + bh + payload)
                lo = hi = 0
                vals = c.data.values if c.variable else c.data
                if vals.size and c.leaf != "TLeafO":
                    lo, hi = vals.min(), vals.max()
                info.append((c, lo, hi, seeks, nbytes, tot, zip_))
            kl = _keylen(big, "TTree", tname, tname)
            w = _W(origin=kl)
            at = w.begin(20)
            w.tnamed(tname, tname)
            w.versioned(2, ">hhh", 602, 1, 1)           # TAttLine
            w.versioned(2, ">hh", 0, 1001)              # TAttFill
            w.versioned(2, ">hhf", 1, 1, 1.0)           # TAttMarker
            tot = sum(x[5] for x in info)
            zip_ = sum(x[6] for x in info)
            w.put(">qqqqqd", n, tot, zip_, zip_, zip_, 1.0)
            w.put(">iiiii", 0, 25, 0, 1000, 0)          # .., fDefaultEntryOffsetLen, fNClusterRange
            w.put(">qqqqqq", 1000000000000, 1000000000000, 0, -300000000, per_basket, 1000000)
            w.put(">BB", 0, 0)                          # fClusterRangeEnd, fClusterSize: none
            w.versioned(1, ">B", 0)                     # fIOFeatures
            leaf_tags = {}
            w.objarray([("TBranchElement" if c.vector else "TBranch",
                         _branch_body(c, lo, hi, nbk, n, bounds, seeks, nb_, tb, zb, fcompress, leaf_tags))
                        for c, lo, hi, seeks, nb_, tb, zb in info])
            w.objarray([("ref", leaf_tags[x[0].name]) for x in info])
            w.put(">I", 0)                              # fAliases
            w.put(">ii", 0, 0)                          # fIndexValues (TArrayD), fIndex (TArrayI): empty
            w.put(">IIII", 0, 0, 0, 0)                  # fTreeIndex, fFriends, fUserInfo, fBranchRef
            w.end(at)
            _, _, khdr = write_key("TTree", tname, tname, bytes(w.b), pdir)
            (dirs[d]["keys"] if d else top_keys).append(khdr)
        # key lists, deepest directory first (a directory's list holds its sub-directories' keys)
        for d in sorted(dirs, key=len, reverse=True):
            rec = dirs[d]
            hdrs = rec["keys"] + [dirs[s]["hdr"] for s in dirs if len(s) == len(d) + 1 and s[:len(d)] == d]
            rec["seek_keys"], rec["nbytes_keys"], _ = write_key("TDirectory", d[-1], "",
                                                                struct.pack(">i", len(hdrs)) + b"".join(hdrs),
                                                                rec["pos"], compress_it=False)
            rec["hdr"] = _key_header(big, rec["keylen"] + 60, 60, rec["keylen"], 1, rec["pos"], seek_dir(d[:-1]),
                                     "TDirectory", d[-1], "", now)
        top_keys += [dirs[s]["hdr"] for s in dirs if len(s) == 1]
        top_seek_keys, top_nbytes_keys, _ = write_key("TFile", fname, title,
                                                      struct.pack(">i", len(top_keys)) + b"".join(top_keys), BEGIN,
                                                      compress_it=False)
        # streamer information: an empty TList
        kl = _keylen(big, "TList", "StreamerInfo", "Doubly linked list")
        w = _W(origin=kl)
        at = w.begin(5)
        w.tobject()
        w.string("")
        w.put(">i", 0)
        w.end(at)
        seek_info, nbytes_info, _ = write_key("TList", "StreamerInfo", "Doubly linked list", bytes(w.b), BEGIN,
                                              compress_it=False)
        # free segments: one, from the end of the file on
        end = pos + _keylen(big, "TFile", fname, title) + (18 if big else 10)
        fr = struct.pack(">hqq", 1001, end, 1 << 62) if big else struct.pack(">hii", 1, end, START_BIG_FILE)
        seek_free, nbytes_free, _ = write_key("TFile", fname, title, fr, BEGIN, compress_it=False)
        if pos != end:
            raise AssertionError("free-segment record size")
        for d, rec in dirs.items():
            f.seek(rec["pos"])
            f.write(rec["hdr"] + _dir_record(big, now, rec["nbytes_keys"], rec["keylen"], rec["pos"],
                                             seek_dir(d[:-1]), rec["seek_keys"], uid))
        f.seek(BEGIN)
        w = _W()
        w.string(fname)
        w.string(title)
        f.write(_key_header(big, top_nbytes, top_nbytes - top_keylen, top_keylen, 1, BEGIN, 0, "TFile", fname, title,
                            now) + bytes(w.b) +
                _dir_record(big, now, top_nbytes_keys, top_keylen + namelen, BEGIN, 0, top_seek_keys, uid))
        f.seek(0)
        h = _W()
        h.b += b"root"
        h.put(">ii", ROOT_VERSION + (1000000 if big else 0), BEGIN)
        if big:
            h.put(">qqiiiBiqi", end, seek_free, nbytes_free, 1, top_keylen + namelen, 8, fcompress, seek_info,
                  nbytes_info)
        else:
            h.put(">iiiiiBiii", end, seek_free, nbytes_free, 1, top_keylen + namelen, 4, fcompress, seek_info,
                  nbytes_info)
        h.put(">h", 1)
        h.b += uid
        f.write(bytes(h.b))
    return path
