"""The version-6 lookup-table reader (crv_lookup_file_info / _read, host memory) against the reference's load
(crv/crvfastsim/response/lookup.py:149-179): identical decoded arrays, dtypes and shapes on a file written by the
reference's own test double and on one with edge cases; the reference's ValueErrors on malformed files.  No GPU."""
import struct

import numpy as np
import pytest

from crvgpu import lookup_file as LF


def _decoded(g, tag):
    return {k[len(tag) + 1:]: g[k] for k in g.files if k.startswith(tag + "_") and k != f"{tag}_image"}


@pytest.mark.parametrize("tag", ["a", "b"])
def test_reader_matches_the_references_load(golden, tag):
    g = golden("lookup_file.npz")
    L = LF.parse(g[f"{tag}_image"].tobytes(), "LookupTable_x")
    ours, ref = LF.arrays(L), _decoded(g, tag)
    assert set(ours) == set(ref)
    for k in ref:
        a, b = np.asarray(ours[k]), ref[k]
        assert a.dtype == b.dtype and a.shape == b.shape and a.tobytes() == b.tobytes(), k


def test_load_reads_files_by_name(golden, tmp_path, monkeypatch):
    g = golden("lookup_file.npz")
    (tmp_path / "LookupTable_2370_1").write_bytes(g["b_image"].tobytes())
    monkeypatch.setenv("CRVFS_LOOKUP_DIR", str(tmp_path))
    L = LF.load("2370_1")
    assert L.name == "LookupTable_2370_1" and L.version == (6, 2) and L.reflector == 1
    assert L.tables["ckfiber"].delays.shape == (0, 1)
    assert LF.load("LookupTable_2370_1", str(tmp_path)).reflector == 1


def _bins_start(image):
    """Byte offset of the first bin record (after header, Cerenkov maps and edges)."""
    o = 12 + 4 + 80
    for _ in range(2 + 7):
        n = struct.unpack_from("<Q", image, o)[0]
        o += 8 + n * (16 if _ < 2 else 8)
    return o


def test_malformed_files_are_refused_like_the_reference(golden):
    img = bytearray(golden("lookup_file.npz")["a_image"].tobytes())
    bad = bytearray(img)
    struct.pack_into("<i", bad, 0, 5)
    with pytest.raises(ValueError, match=r"lookup table version 5\.0, expected 6\.x"):
        LF.parse(bytes(bad))
    bad = bytearray(img)
    b0 = _bins_start(img)
    nd = struct.unpack_from("<Q", img, b0 + 8)[0]
    ne = struct.unpack_from("<Q", img, b0 + 16 + nd)[0]
    struct.pack_into("<I", bad, b0 + 24 + nd + ne, 7)            # the second bin claims to be bin 7
    with pytest.raises(ValueError, match="corrupt lookup table: bin 7 at position 1"):
        LF.parse(bytes(bad))
    with pytest.raises(ValueError, match="3 trailing bytes"):
        LF.parse(bytes(img) + b"\0\0\0")
    for cut in (1, 50, len(img) // 2, len(img) - 40):
        with pytest.raises(ValueError, match="truncated"):
            LF.parse(bytes(img[:cut]))
    with pytest.raises(ValueError, match="truncated"):
        LF.parse(b"")


def test_empty_edge_vectors_and_absurd_sizes_are_refused():
    head = struct.pack("<3i4x", 6, 0, 0) + np.zeros(10, "<f8").tobytes() + struct.pack("<Q", 0) * 2
    edges = b"".join(struct.pack("<Q", 2) + np.array([0.0, 1.0], "<f8").tobytes() for _ in range(6))
    with pytest.raises(ValueError, match="empty bin-edge vector 'r'"):
        LF.parse(head + edges + struct.pack("<Q", 0))
    big = b"".join(struct.pack("<Q", 1001) + np.arange(1001, dtype="<f8").tobytes() for _ in range(7))
    with pytest.raises(ValueError, match="table sizes beyond the file"):
        LF.parse(head + big)
    with pytest.raises(ValueError, match="truncated"):
        LF.parse(head + struct.pack("<Q", 1 << 62))


def test_a_read_table_drives_the_propagation_fits_like_the_references(golden):
    """The reader's table in the lookup model's host setup: table_propagation gives what it gives on the reference's
    decoded arrays."""
    from crvgpu.lookup import table_propagation
    g = golden("lookup_file.npz")
    L = LF.parse(g["a_image"].tobytes())
    ref = _decoded(g, "a")
    R = LF.LookupTable("ref", tuple(ref["version"]), int(ref["reflector"]), *ref["constants"], ref["ck_scint"],
                       ref["ck_fiber"], {k: ref[f"edges_{k}"] for k in LF.EDGES},
                       {t: LF.Table(*(ref[f"{t}_{f}"] for f in ("prob", "delays", "delay_sum", "emis", "emis_sum")))
                        for t in LF.TABLES})
    assert np.array_equal(np.asarray(table_propagation(L)), np.asarray(table_propagation(R)))


def _mutate(image, recipe):
    """The recipes of make_golden.py lookup_fuzz: set bytes, cut, insert, delete."""
    b = bytearray(image)
    for op in recipe:
        if op[0] == "set":
            b[op[1]:op[1] + len(op[2])] = bytes(op[2])
        elif op[0] == "cut":
            b = b[:op[1]]
        elif op[0] == "ins":
            b = b[:op[1]] + bytes(op[2]) + b[op[1]:]
        else:
            b = b[:op[1]] + b[op[1] + op[2]:]
    return bytes(b)


def _decoded_hash(arrays):
    import hashlib
    h = hashlib.sha256()
    for k in sorted(arrays):
        a = np.ascontiguousarray(arrays[k])
        h.update(f"{k}|{a.dtype.str}|{a.shape}|".encode())
        h.update(a.tobytes())
    return h.hexdigest()


def test_mutated_files_get_the_references_verdict(golden):
    """600 mutated images (make_golden.py lookup_fuzz): where the reference's load decodes one, this reader decodes the
    same arrays (same content hash); where it fails (ValueError, or OverflowError / IndexError / MemoryError from
    absurd length fields), this reader raises ValueError.  No image crashes the native parser."""
    import json
    import os
    g = golden("lookup_file.npz")
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lookup_fuzz.json")) as f:
        cases = json.load(f)
    assert len(cases) == 600
    decoded = 0
    for i, c in enumerate(cases):
        image = _mutate(g[f"{c['image']}_image"].tobytes(), c["recipe"])
        if c["verdict"].startswith("error:"):
            with pytest.raises(ValueError):
                LF.parse(image)
        else:
            assert _decoded_hash(LF.arrays(LF.parse(image))) == c["verdict"], i
            decoded += 1
    assert decoded >= 50
