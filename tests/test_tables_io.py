"""Step-table I/O (core/mu2efastsim/tables.py, crv/crvfastsim/tables.py) on the CPU: the ROOT layer (crvgpu.rootio)
round-trips every leaf type through uncompressed, zlib, LZMA and LZ4 baskets; the file's records are consistent (the
header's end and seeks, the key list, the basket byte counts, the tree's leaf references resolving to the branches'
leaves); the native LZ4 and XXH64 decoders meet their published test values and refuse malformed blocks; and the
tables helpers (read, read_many, livetime, primary_muons, all_primary_muons, primary_muon_crossings, write in both
forms) give what the reference's pandas code gives, restated here with plain loops.

Parity with uproot/ROOT themselves is not pinned: neither is installed here and the reference ships no ROOT files.
"""
import os
import struct

import numpy as np
import pytest

from crvgpu import rootio as R
from crvgpu import tables as TB


# ---- a greedy LZ4 block compressor (test side only), to make "L4" baskets the native decoder must read

def _lz4_len(out, v):
    while v >= 255:
        out.append(255)
        v -= 255
    out.append(v)


def _lz4_compress(data):
    out, table, i, anchor, n = bytearray(), {}, 0, 0, len(data)

    def seq(lit, off=None, m=0):
        tok_l = min(len(lit), 15)
        tok_m = 0 if off is None else min(m - 4, 15)
        out.append((tok_l << 4) | tok_m)
        if len(lit) >= 15:
            _lz4_len(out, len(lit) - 15)
        out.extend(lit)
        if off is not None:
            out.extend(off.to_bytes(2, "little"))
            if m - 4 >= 15:
                _lz4_len(out, m - 4 - 15)

    while i + 4 <= n - 5:
        key = bytes(data[i:i + 4])
        j = table.get(key)
        table[key] = i
        if j is not None and i - j <= 65535:
            m = 4
            while i + m < n - 5 and data[j + m] == data[i + m]:
                m += 1
            seq(data[anchor:i], i - j, m)
            i += m
            anchor = i
        else:
            i += 1
    seq(data[anchor:])
    return bytes(out)


def _l4_blocks(raw):
    from crvgpu import _capi
    L = _capi.load()
    out = []
    for a in range(0, len(raw), R.MAX_BLOCK):
        chunk = raw[a:a + R.MAX_BLOCK]
        body = _lz4_compress(chunk)
        body = L.crv_xxh64(body, len(body), 0).to_bytes(8, "big") + body
        out.append(R._block(b"L4", 1, chunk, body))
    z = b"".join(out)
    return z if len(z) < len(raw) else None


def _columns(n, rng):
    return {"run": np.full(n, 1400, np.uint32), "subrun": rng.integers(0, 9, n).astype(np.uint32),
            "event": np.arange(n, dtype=np.uint32), "bar": rng.integers(0, 5000, n).astype(np.int32),
            "t0": rng.uniform(0, 1e3, n), "edep": rng.uniform(0, 5, n).astype(np.float32),
            "big": rng.integers(-2 ** 62, 2 ** 62, n), "u64": rng.integers(0, 2 ** 63, n).astype(np.uint64),
            "flag": rng.random(n) < 0.3, "s": rng.integers(-300, 300, n).astype(np.int16),
            "us": rng.integers(0, 60000, n).astype(np.uint16), "c": rng.integers(-100, 100, n).astype(np.int8),
            "uc": rng.integers(0, 255, n).astype(np.uint8), "pos": rng.normal(size=(n, 3)),
            "rep": np.repeat(np.arange(n // 50 + 1), 50)[:n].astype(np.int64)}


@pytest.mark.parametrize("mode", ["none", "zlib", "lzma", "lz4"])
def test_every_leaf_type_round_trips(tmp_path, mode):
    rng = np.random.default_rng(1)
    cols = _columns(30011, rng)
    path = str(tmp_path / f"a_{mode}.root")
    kw = dict(none=dict(compression=0), zlib=dict(compression=101), lzma=dict(compression=205),
              lz4=dict(compression=404, _compressor=_l4_blocks))[mode]
    R.write(path, {"dump/steps": cols, "dump/sub/x": {"v": np.arange(10.0)}, "top": {"k": np.arange(5, dtype=np.int32)},
                   "dump/empty": {"e": np.zeros(0)}, "dump/none": None}, basket_bytes=16384, **kw)
    with R.RootFile(path) as f:
        assert f.keys() == ["top", "dump", "dump/steps", "dump/sub", "dump/sub/x"]
        T = f["dump/steps"]
        assert len(T) == 30011 and T.keys() == list(cols)
        assert T.branches["bar"].write_basket > 10                 # several baskets per branch
        got = T.arrays()
        for k, v in cols.items():
            assert got[k].dtype == v.dtype and got[k].shape == v.shape and np.array_equal(got[k], v), k
        assert np.array_equal(f["dump/sub/x"].arrays()["v"], np.arange(10.0))
        assert list(f["top"].arrays(["k"])) == ["k"]
        assert T.branches["pos"].title == "pos[3]/D" and T.branches["us"].title == "us/s"
        assert f.compression == (0 if mode == "none" else kw["compression"])
        with pytest.raises(KeyError):
            f["dump/nothing"]
        with pytest.raises(KeyError):
            T.arrays(["nothing"])


def test_file_records_are_consistent(tmp_path):
    """Header, key list, basket byte counts and the tree's leaf references, read back from the raw bytes."""
    path = str(tmp_path / "c.root")
    rng = np.random.default_rng(2)
    R.write(path, {"dump/steps": _columns(5000, rng)}, basket_bytes=8192)
    raw = open(path, "rb").read()
    assert raw[:4] == b"root"
    version, begin, end, seek_free, nbytes_free, nfree, nbytes_name, units, comp, seek_info, nbytes_info = \
        struct.unpack_from(">iiiiiiiBiii", raw, 4)
    assert version == R.ROOT_VERSION and begin == 100 and end == len(raw) and units == 4 and comp == 101
    assert seek_free + nbytes_free == end and nfree == 1
    with R.RootFile(path) as f:
        k = R._key(R._Cursor(f.buf, seek_info))
        assert (k.classname, k.name, k.nbytes) == ("TList", "StreamerInfo", nbytes_info)
        top = R._key(R._Cursor(f.buf, begin))
        assert top.classname == "TFile" and nbytes_name == top.keylen + 2 + len(top.name) + len(top.title)
        T = f["dump/steps"]
        leaves = [b.leaves[0] for b in T.branches.values()]
        assert T.leaves is not None and len(T.leaves) == len(leaves)
        assert all(a is b for a, b in zip(T.leaves, leaves))       # references resolve to the branches' leaves
        for b in T.branches.values():
            for i in range(b.write_basket):
                bk = R._key(R._Cursor(f.buf, int(b.basket_seek[i])))
                assert bk.classname == "TBasket" and bk.name == b.name and bk.title == "steps"
                assert bk.nbytes == b.basket_bytes[i] and bk.seek_key == b.basket_seek[i]
            assert b.basket_entry[b.write_basket] == 5000 and not b.basket_seek[b.write_basket]


def test_big_file_layout_reads_back(tmp_path, monkeypatch):
    """The 64-bit layout (file version + 1000000, key version 1004, directory version 1005), forced on a small file."""
    monkeypatch.setattr(R, "START_BIG_FILE", 0)
    path = str(tmp_path / "big.root")
    rng = np.random.default_rng(3)
    cols = _columns(3000, rng)
    R.write(path, {"dump/steps": cols}, basket_bytes=4096)
    raw = open(path, "rb").read()
    assert struct.unpack_from(">i", raw, 4)[0] == R.ROOT_VERSION + 1000000
    with R.RootFile(path) as f:
        got = f["dump/steps"].arrays()
        assert f.get_key("dump/steps").version == 1004
    for k, v in cols.items():
        assert np.array_equal(got[k], v), k


def test_xxh64_and_lz4_decoders():
    from crvgpu import _capi
    L = _capi.load()
    assert L.crv_xxh64(b"", 0, 0) == 0xEF46DB3751D8E999          # published XXH64 test values
    assert L.crv_xxh64(b"abc", 3, 0) == 0x44BC2CF5AD770999
    rng = np.random.default_rng(4)
    data = bytes(rng.integers(0, 4, 40000).astype(np.uint8)) + b"abcd" * 3000 + bytes(rng.integers(0, 256, 5000)
                                                                                    .astype(np.uint8)) + b"\0" * 70000
    blocks = _l4_blocks(data)
    assert blocks is not None and len(blocks) < len(data) // 2
    assert R.decompress(blocks, len(data)) == data
    # malformed blocks: negative status, nothing written past the output buffer
    import ctypes
    body = _lz4_compress(data)
    out = ctypes.create_string_buffer(len(data) + 16)
    assert L.crv_lz4_block_decompress(body, len(body), out, len(data)) == len(data)
    assert L.crv_lz4_block_decompress(body, len(body), out, len(data) - 1) < 0        # output too small
    assert L.crv_lz4_block_decompress(body[:len(body) // 2], len(body) // 2, out, len(data)) != len(data)
    i, lit = 1, body[0] >> 4                                    # the first sequence's match offset -> 0
    if lit == 15:
        while body[i] == 255:
            lit += 255
            i += 1
        lit += body[i]
        i += 1
    bad = bytearray(body)
    bad[i + lit] = bad[i + lit + 1] = 0
    assert L.crv_lz4_block_decompress(bytes(bad), len(bad), out, len(data)) < 0
    # a wrong checksum is refused
    b2 = bytearray(blocks)
    b2[9] ^= 1
    with pytest.raises(R.RootFormatError):
        R.decompress(bytes(b2), len(data))


def test_mixed_blocks_and_refusals():
    raw = bytes(range(256)) * 400
    z = R._block(b"ZL", 8, raw[:50000], __import__("zlib").compress(raw[:50000])) + \
        R._block(b"XZ", 0, raw[50000:], __import__("lzma").compress(raw[50000:]))
    assert R.decompress(z, len(raw)) == raw
    with pytest.raises(R.RootFormatError, match="zstd"):
        R.decompress(R._block(b"ZS", 1, b"x" * 10, b"0123"), 10)
    with pytest.raises(R.RootFormatError):
        R.decompress(b"ZL\x08\xff\x00\x00", 10)


def test_not_a_root_file(tmp_path):
    p = tmp_path / "x.root"
    p.write_bytes(b"root")
    with pytest.raises(R.RootFormatError):
        R.RootFile(str(p))
    p.write_bytes(b"notroot" * 20)
    with pytest.raises(R.RootFormatError):
        R.RootFile(str(p))


def test_unsupported_columns_are_refused(tmp_path):
    with pytest.raises(TypeError):
        R.write(str(tmp_path / "u.root"), {"t": {"s": np.array(["a", "b"])}})
    with pytest.raises(ValueError):
        R.write(str(tmp_path / "u.root"), {"t": {"a": np.zeros(3), "b": np.zeros(4)}})


# ---- the tables API against the reference's pandas semantics, restated with loops

def _dumper_tables(rng, n_events=40):
    steps, parts, gen = {k: [] for k in ("run", "subrun", "event", "nstep", "bar", "sp", "t0", "t1", "edep",
                                         "x0", "y0", "z0", "x1", "y1", "z1", "len")}, \
        {k: [] for k in ("run", "subrun", "event", "key", "parent", "pdg", "isprim")}, \
        {k: [] for k in ("run", "subrun", "event", "idx", "pdg", "x")}
    for e in range(n_events):
        sub = 1 + e // 15
        nmu = rng.integers(0, 3)
        for g in range(rng.integers(1, 4)):
            pdg = 13 if g < nmu else rng.choice([11, 22, -13])
            for k, v in (("run", 1), ("subrun", sub), ("event", e), ("idx", 2 - g), ("pdg", pdg), ("x", rng.normal())):
                gen[k].append(v)
        keys = [1, 2, 5]
        for kk in keys:
            for k, v in (("run", 1), ("subrun", sub), ("event", e), ("key", kk), ("parent", -1 if kk == 1 else 1),
                         ("pdg", 13 if kk == 1 else rng.choice([11, 13])), ("isprim", int(kk == 1))):
                parts[k].append(v)
        ns = rng.integers(0, 12)
        for s in range(ns):
            vals = dict(run=1, subrun=sub, event=e, nstep=ns, bar=rng.integers(0, 6), sp=rng.choice(keys),
                        t0=rng.uniform(0, 100), edep=rng.uniform(0, 3), len=rng.uniform(1, 20))
            vals["t1"] = vals["t0"] + 0.5
            for a in "xyz":
                vals[f"{a}0"], vals[f"{a}1"] = rng.normal(), rng.normal()
            for k in steps:
                steps[k].append(vals[k])
    dt = dict(run=np.uint32, subrun=np.uint32, event=np.uint32, nstep=np.int32, bar=np.int32, sp=np.int32,
              t0=np.float64, t1=np.float64, key=np.int32, parent=np.int32, pdg=np.int32, isprim=np.int32,
              idx=np.int32, x=np.float64)
    conv = lambda d: {k: np.asarray(v, dt.get(k, np.float32)) for k, v in d.items()}  # noqa: E731
    return conv(steps), conv(parts), conv(gen)


def test_tables_api_matches_the_reference_semantics(tmp_path, capsys):
    rng = np.random.default_rng(7)
    steps, parts, gen = _dumper_tables(rng)
    subruns = {"run": np.array([1, 1, 1, 1], np.uint32), "subrun": np.array([1, 2, 2, 3], np.uint32),
               "livetime": np.array([1.5, 2.0, 2.0, 0.25]), "primaries": np.array([10, 20, 20, 3], np.uint64)}
    p1, p2 = str(tmp_path / "crvsteps.1.root"), str(tmp_path / "crvsteps.2.root")
    TB.write(p1, steps, parts, gen=gen, subruns=subruns, as_ttree=True)        # crv form
    TB.write(p2, {"steps": steps, "particles": parts, "subruns": subruns})      # core form
    assert "wrote" in capsys.readouterr().out
    s = TB.read(p1, "steps", library="np")
    assert isinstance(s, TB.StepRows) and len(s) == len(steps["bar"]) and s.bar is s["bar"]
    for k, v in steps.items():
        assert s[k].dtype == v.dtype and np.array_equal(s[k], v), k
    both = TB.read_many([str(tmp_path / "crvsteps.*.root")], "steps", ["event", "bar"], library="np")
    assert list(both) == ["event", "bar"] and np.array_equal(both["bar"], np.r_[steps["bar"], steps["bar"]])
    # livetime: each (run, subrun) once over both files
    assert TB.livetime([p1, p2]) == pytest.approx(1.5 + 2.0 + 0.25)
    # primary_muons: first |pdg| == 13 row of each event
    pm = TB.primary_muons(gen)
    want, seen = [], set()
    for i in range(len(gen["pdg"])):
        key = (gen["run"][i], gen["subrun"][i], gen["event"][i])
        if abs(gen["pdg"][i]) == 13 and key not in seen:
            seen.add(key)
            want.append(i)
    assert np.array_equal(pm["x"], gen["x"][want])
    # all_primary_muons: ordered by (run, subrun, event, idx), mukey = 1, 2, ...
    am = TB.all_primary_muons(gen)
    rows = sorted([i for i in range(len(gen["pdg"])) if abs(gen["pdg"][i]) == 13],
                  key=lambda i: (gen["run"][i], gen["subrun"][i], gen["event"][i], gen["idx"][i]))
    assert np.array_equal(am["x"], gen["x"][rows])
    mk, cnt = [], {}
    for i in rows:
        key = (gen["run"][i], gen["subrun"][i], gen["event"][i])
        cnt[key] = cnt.get(key, 0) + 1
        mk.append(cnt[key])
    assert np.array_equal(am["mukey"], mk)
    # primary_muon_crossings: inner merge on (run, subrun, event, sp = primary muon key), groups in first-seen order
    sector_of_bar = np.array([0, 0, 1, 1, 2, 2])
    cx = TB.primary_muon_crossings(s, TB.read(p1, "particles", library="np"), sector_of_bar)
    with pytest.raises(ValueError):
        TB.read(p1, "steps", library="arrow")
    assert TB._library(None) in ("np", "pd")
    prim = {(parts["run"][i], parts["subrun"][i], parts["event"][i], parts["key"][i])
            for i in range(len(parts["key"])) if parts["isprim"][i] == 1 and abs(parts["pdg"][i]) == 13}
    groups = {}
    for i in range(len(steps["bar"])):
        if (steps["run"][i], steps["subrun"][i], steps["event"][i], steps["sp"][i]) in prim:
            g = (steps["run"][i], steps["subrun"][i], steps["event"][i], steps["bar"][i])
            e = groups.setdefault(g, [0.0, 0.0, np.inf, 0])
            e[0] += float(steps["edep"][i])
            e[1] += float(steps["len"][i])
            e[2] = min(e[2], steps["t0"][i])
            e[3] += 1
    assert len(groups) > 10 and len(cx) == len(groups)
    assert [tuple(int(cx[k][j]) for k in ("run", "subrun", "event", "bar")) for j in range(len(cx))] == \
        [tuple(int(x) for x in g) for g in groups]
    v = np.array(list(groups.values()))
    np.testing.assert_allclose(cx["edep"], v[:, 0], rtol=1e-6)
    np.testing.assert_allclose(cx["len"], v[:, 1], rtol=1e-6)
    assert np.array_equal(cx["t0"], v[:, 2]) and np.array_equal(cx["nsteps"], v[:, 3])
    assert np.array_equal(cx["sector"], sector_of_bar[cx["bar"]])
    assert TB.expand([str(tmp_path / "none.*.root")]) == [str(tmp_path / "none.*.root")]
    assert os.path.getsize(p1) > 0


def test_step_table_feeds_the_engine_host_path(tmp_path):
    """A dumper-layout steps tree read back goes into the engine's step upload as it is: midpoints from the start/end
    columns (as the oracle's step frame takes them) and events keyed by (subrun, event)."""
    from crvgpu import geometry as GM
    from crvgpu.response import _col
    rng = np.random.default_rng(8)
    steps, parts, gen = _dumper_tables(rng, 60)
    p = str(tmp_path / "s.root")
    TB.write(p, steps, parts)
    s = TB.read(p, "steps", library="np")
    assert np.array_equal(GM.event_key(s), (steps["subrun"].astype(np.int64) << 20) | steps["event"])
    for a in "xyzt":
        assert np.array_equal(_col(s, a), 0.5 * (steps[f"{a}0"].astype(float) + steps[f"{a}1"].astype(float))), a


def test_jagged_columns_round_trip(tmp_path):
    """Counted arrays (n<name> counter + name[n<name>], as uproot writes them) and std::vector element branches (the
    art dumper's layout), through every basket split and compression."""
    rng = np.random.default_rng(9)
    n = 4001
    adc = R.JaggedArray.from_rows([rng.integers(-50, 4000, rng.integers(0, 30)).astype(np.int16) for _ in range(n)],
                                  np.int16)
    volt = R.JaggedArray.from_rows([rng.normal(size=rng.integers(0, 5)) for _ in range(n)], np.float64)
    cols = {"event": np.arange(n, dtype=np.uint32), "adc": adc, "x": rng.normal(size=n), "volt": volt,
            "wfidx": [np.arange(i % 3, dtype=np.int32) for i in range(n)]}
    for comp, vec in ((0, ()), (101, ()), (101, ("adc", "volt", "wfidx"))):
        p = str(tmp_path / f"j{comp}{len(vec)}.root")
        R.write(p, {"crvdump/digis": cols}, compression=comp, basket_bytes=2048, _vectors=vec)
        with R.RootFile(p) as f:
            T = f["crvdump/digis"]
            got = T.arrays()
            if not vec:
                assert T.keys() == ["event", "nadc", "adc", "x", "nvolt", "volt", "nwfidx", "wfidx"]
                b = T.branches["adc"]
                assert b.title == "adc[nadc]/S" and b.leaves[0].leaf_count.name == "nadc"
                assert np.array_equal(got["nadc"], adc.counts)
            else:
                assert T.branches["adc"].cls == "TBranchElement" and T.branches["adc"].class_name == "vector<short>"
            assert T.branches["adc"].write_basket > 5
        assert got["adc"] == adc and got["volt"] == volt and np.array_equal(got["x"], cols["x"])
        assert got["wfidx"].tolist() == [list(range(i % 3)) for i in range(n)]


def test_reco_tables_feed_the_pulse_fit_grouping(tmp_path):
    """crvdump/digis + calib written from the oracle's digis read back through reftables (read, calib, conditions,
    event_key) and grouped by reftables.waveforms give the oracle's reco waveforms; the art dumper's vector layout of
    the same digis reads back the same; Conditions.from_csv reads the calib columns."""
    from crvgpu import reftables as RT
    from crvgpu.config import Conditions
    from oracle import oracle as O
    from tests.test_chain_glue_host import _digis
    D, cond = _digis()
    cond.status[[5, 9]] = [2, 1]
    path = str(tmp_path / "crvdump.root")
    dig = RT.digis_table(D, cond, run=1400)
    RT.write(path, {"digis": dig, "calib": RT.calib_table(cond)})
    d = RT.read([path], "digis")
    assert np.array_equal(d["adc"].values, np.asarray(D["adc"]).reshape(-1)) and np.all(d["adc"].counts == 12)
    assert np.array_equal(RT.event_key(d) & ((1 << 40) - 1), np.asarray(D["chan"]) // 32768)
    c = RT.conditions(path)
    assert np.array_equal(c.pedestal, np.asarray(cond.pedestal, np.float32)) and np.array_equal(c.status, cond.status)
    W = RT.waveforms(path)
    Wo = O.reco_waveforms(D, cond)
    keep = ~((np.asarray(cond.status)[Wo["chan"]] >> 1) & 1).astype(bool)
    assert keep.sum() < len(keep)                                  # the ignored channel's waveforms are dropped
    for k in ("bar", "sipm", "adc", "n", "start"):
        assert np.array_equal(np.asarray(W[k]), np.asarray(Wo[k])[keep]), k
    assert np.array_equal(W["ev"] & ((1 << 40) - 1), np.asarray(Wo["ev"])[keep])
    np.testing.assert_array_equal(W["ped"], np.asarray(cond.pedestal, np.float32)[W["chan"]])
    # the art dumper's layout: std::vector ADC branches
    vpath = str(tmp_path / "crvdump_vec.root")
    R.write(vpath, {"crvdump/digis": dig, "crvdump/calib": RT.calib_table(cond)}, _vectors=("adc",))
    dv = RT.read(vpath, "digis")
    assert dv["adc"] == d["adc"] and set(d) - set(dv) == {"nadc"}
    Wv = RT.waveforms(vpath)
    assert all(np.array_equal(np.asarray(Wv[k]), np.asarray(W[k])) for k in W)
    # Conditions.from_csv on the calib columns
    csv = tmp_path / "calib.csv"
    rows = np.c_[np.arange(len(cond.pedestal)), cond.pedestal, cond.pulsearea, cond.pulseheight, cond.timeoffset,
                 cond.status, cond.roc, cond.feb, np.zeros(len(cond.pedestal))]
    np.savetxt(csv, rows, delimiter=",", fmt="%.17g")
    cc = Conditions.from_csv(str(csv))
    for k in ("pedestal", "pulsearea", "pulseheight", "timeoffset", "status", "roc", "feb"):
        assert np.array_equal(getattr(cc, k), np.asarray(getattr(cond, k))), k


def test_truncated_and_corrupted_files_are_refused(tmp_path):
    """A file cut short or with a damaged basket raises RootFormatError (or KeyError for a missing tree); the reader
    never reads outside the file."""
    rng = np.random.default_rng(11)
    p = str(tmp_path / "t.root")
    R.write(p, {"dump/steps": _columns(20000, rng)}, basket_bytes=8192)
    raw = open(p, "rb").read()
    with R.RootFile(p) as f:
        b = f["dump/steps"].branches["t0"]
        seek = int(b.basket_seek[1])
        k = R._key(R._Cursor(f.buf, seek))
    bad = bytearray(raw)
    for i in range(seek + k.keylen + 20, seek + k.keylen + 60):
        bad[i] ^= 0x5A
    q = str(tmp_path / "bad.root")
    open(q, "wb").write(bytes(bad))
    with R.RootFile(q) as f:
        with pytest.raises(R.RootFormatError):
            f["dump/steps"].arrays(["t0"])
        with R.RootFile(p) as g:                              # other branches still read
            assert np.array_equal(f["dump/steps"].arrays(["bar"])["bar"], g["dump/steps"].arrays(["bar"])["bar"])
    for cut in (len(raw) // 2, len(raw) - 200, 150):
        c = str(tmp_path / f"cut{cut}.root")
        open(c, "wb").write(raw[:cut])
        with pytest.raises((R.RootFormatError, KeyError)):
            with R.RootFile(c) as f:
                f["dump/steps"].arrays()


def test_cluster_and_event_trees_of_the_chain_outputs(tmp_path):
    """reftables.clusters_table / events_table on the chain's cluster output (here the oracle's, in the same detail
    format as chain.clusters(..., detail=True)): member pulses and layers per cluster (the reference finder's `pulses`
    and `layers`), the per-event index, and a round trip through a crvdump file with jagged columns."""
    from crvgpu import config as CF
    from crvgpu import geometry as GM
    from crvgpu import reftables as RT
    from oracle import oracle as O
    from tests.test_chain_glue_host import _digis
    D, cond = _digis()
    W = O.reco_waveforms(D, cond)
    rcfg = CF.RecoConfig()
    geom = GM.module_geometry()
    G = GM.sector_geom(geom)
    out = O.clusters_from_pulses(W, O.pulses_from_waveforms(W, cond, rcfg, rcfg.period), G, cond.status,
                                 CF.workload_finder(G.sector_names))
    n = len(out["cl_event"])
    assert n >= 2
    t = RT.clusters_table(out, G, run=1400)
    for c in range(n):
        assert t["pulses"][c].tolist() == list(out["mem_idx"][out["mem_cl"] == c])
        assert t["layers"][c].tolist() == out["cl_layers"][c]
    ev = np.asarray(out["cl_event"])
    assert np.array_equal(t["idx"], [int(np.sum(ev[:i] == ev[i])) for i in range(n)])
    uev, ncl = np.unique(ev, return_counts=True)
    e = RT.events_table(uev, run=1400, ncluster=ncl, npulse={int(k): 1 for k in uev})
    p = str(tmp_path / "crvdump_cl.root")
    RT.write(p, {"clusters": t, "events": e})
    r = RT.read(p, "clusters")
    for k, v in t.items():
        assert (r[k] == v) if isinstance(v, R.JaggedArray) else np.array_equal(r[k], v), k
    re_ = RT.read(p, "events")
    assert np.array_equal(re_["ncluster"], ncl) and np.all(re_["spill"] == -1) and np.all(re_["npulse"] == 1)
    assert np.array_equal(RT.event_key(r) & ((1 << 40) - 1), ev) and np.all(np.asarray(r["run"]) == 1400)


def test_pulses_tree_from_dumped_digis(tmp_path):
    """reftables.pulses_table on reco waveforms grouped from a dumped digi table and their pulses: one row per pulse in
    (event, waveform, sequence) order, flags bit 0 = failed fit, wfidx = the waveform's digis, and the reference
    reco's reading of it (bar, sipm, seq, pe, time, failed = flags & 1, the first wfidx) gives the pulses back."""
    from crvgpu import config as CF
    from crvgpu import reftables as RT
    from oracle import oracle as O
    from tests.test_chain_glue_host import _digis
    D, cond = _digis()
    path = str(tmp_path / "d.root")
    RT.write(path, {"digis": RT.digis_table(D, cond, run=7), "calib": RT.calib_table(cond)})
    W = RT.waveforms(path)
    rcfg = CF.RecoConfig()
    P = O.reconstruct_full(W["adc"], W["n"], W["start"], W["ped"], W["area"], W["height"], rcfg, rcfg.period)
    t = RT.pulses_table(W, P, run=7)
    assert len(t["pe"]) == len(P["pe"]) > 20
    RT.write(str(tmp_path / "p.root"), {"pulses": t})
    r = RT.read(str(tmp_path / "p.root"), "pulses")
    o = np.lexsort((P["seq"], P["wf"], np.asarray(W["ev"])[P["wf"]]))
    assert np.array_equal(r["pe"], np.asarray(P["pe"])[o].astype(np.float32))
    assert np.array_equal(r["time"], np.asarray(P["time"])[o])
    assert np.array_equal(r["flags"] & 1, np.asarray(P["failed"])[o].astype(np.int32))
    wf = np.asarray(P["wf"])[o]
    assert np.array_equal(r["bar"] * 4 + r["sipm"], np.asarray(W["chan"])[wf])
    first = np.array([row[0] for row in r["wfidx"].tolist()])
    assert np.array_equal(first, np.asarray(W["digi0"])[wf])
    assert np.array_equal(r["wfidx"].counts, -(-np.asarray(W["n"])[wf] // 12))
    assert np.array_equal(RT.event_key(r), np.asarray(W["ev"])[wf])


def test_dataframes_where_pandas_is_installed(tmp_path):
    """With pandas importable, read gives the reference's DataFrame (same columns and values)."""
    pd = pytest.importorskip("pandas")
    rng = np.random.default_rng(3)
    steps, parts, gen = _dumper_tables(rng, 20)
    p = str(tmp_path / "pd.root")
    TB.write(p, steps, parts, gen=gen)
    df = TB.read(p, "steps")
    assert isinstance(df, pd.DataFrame) and list(df.columns) == list(steps)
    for k, v in steps.items():
        assert np.array_equal(df[k].to_numpy(), v), k


def test_mutated_files_fail_cleanly(tmp_path):
    """300 random mutations (byte flips, 1-8 bytes anywhere, zlib and LZ4 baskets): reading either gives the
    original columns or raises RootFormatError / KeyError / ValueError; nothing crashes the process or reads outside
    the file (the native LZ4 decoder checks every length, and its blocks carry a checksum)."""
    rng = np.random.default_rng(21)
    cols = {"a": rng.integers(0, 1000, 3000).astype(np.int32), "b": rng.normal(size=3000),
            "j": R.JaggedArray.from_rows([rng.integers(0, 9, rng.integers(0, 5)).astype(np.int16) for _ in range(3000)],
                                         np.int16)}
    for mode, kw in (("zlib", dict(compression=101)), ("lz4", dict(compression=404, _compressor=_l4_blocks))):
        p = str(tmp_path / f"m_{mode}.root")
        R.write(p, {"dump/t": cols}, basket_bytes=4096, **kw)
        raw = open(p, "rb").read()
        for k in range(150):
            bad = bytearray(raw)
            for _ in range(int(rng.integers(1, 9))):
                bad[int(rng.integers(0, len(raw)))] ^= int(rng.integers(1, 256))
            q = str(tmp_path / "mut.root")
            open(q, "wb").write(bytes(bad))
            try:
                with R.RootFile(q) as f:
                    got = f["dump/t"].arrays()
            except (R.RootFormatError, KeyError, ValueError):
                continue
            assert got["a"].shape == cols["a"].shape and got["b"].dtype == cols["b"].dtype
            assert len(got["j"]) == len(cols["j"])


def test_against_uproot_where_installed(tmp_path):
    """Parity with the reference's ROOT library where it is installed (not in this image): a file written here reads
    the same through uproot, and TTrees uproot writes (flat columns, counted arrays) read the same here."""
    uproot = pytest.importorskip("uproot")
    rng = np.random.default_rng(12)
    n = 5000
    cols = {"run": np.full(n, 1400, np.uint32), "event": np.arange(n, dtype=np.uint32),
            "bar": rng.integers(0, 5000, n).astype(np.int32), "t0": rng.uniform(0, 1e3, n),
            "edep": rng.uniform(0, 5, n).astype(np.float32), "flag": rng.random(n) < 0.5}
    ours = str(tmp_path / "ours.root")
    R.write(ours, {"dump/steps": cols}, basket_bytes=4096)
    with uproot.open(ours) as f:
        got = f["dump/steps"].arrays(library="np")
    for k, v in cols.items():
        assert np.array_equal(got[k], v), k
    theirs = str(tmp_path / "theirs.root")
    counts = rng.integers(0, 6, n)
    jag = [rng.integers(-9, 9, c).astype(np.int16) for c in counts]
    with uproot.recreate(theirs) as f:
        f.mktree("dump/steps", {k: v.dtype for k, v in cols.items()})
        f["dump/steps"].extend(cols)
        import awkward as ak
        f["crvdump/digis"] = {"adc": ak.Array([list(a) for a in jag])}
    with R.RootFile(theirs) as f:
        got = f["dump/steps"].arrays()
        adc = f["crvdump/digis"].arrays()["adc"]
    for k, v in cols.items():
        assert np.array_equal(got[k], v), k
    assert adc.tolist() == [a.tolist() for a in jag]
