"""Warm-start snapshot host logic, no GPU: cache keys, AoA buckets and the
flag hash against the reference's own values (golden vectors from
src/sim/snapshot.cpp), the FCS1 reader and writer against a file written by
the reference, its rejections, and the LRU disk cache (directory scan,
budget eviction oldest-first, hit refresh, protected newest entry,
temporary-file writes, background writer)."""
import os
import time

import numpy as np
import pytest


@pytest.fixture(scope="module")
def sn(built_lib):
    from foil_cfd_gb300 import snapshot
    return snapshot


def test_keys_buckets_and_flag_hash_match_reference(sn, golden, mg):
    g = golden("snapshot")
    for i, (gid, bucket, u, dims, ver) in enumerate(mg.SNAPSHOT_KEYS):
        k = sn.SnapshotKey(gid, bucket, u, dims, ver)
        assert k.hash() == int(g["key_hash"][i]), gid
        assert str(k) == str(g["key_name"][i])
    assert [sn.aoa_bucket(float(a)) for a in g["aoa"]] == list(g["aoa_bucket"])
    assert sn.hash_flags(g["flags"]) == int(g["flags_hash"])


def test_fcs1_reader_and_writer_match_reference_bytes(sn, golden, mg, tmp_path):
    g = golden("snapshot")
    src = tmp_path / "ref.fcs"
    src.write_bytes(g["fcs"].tobytes())
    c = sn.CompactSnapshot()
    c.load(src)
    assert c.has_data and c.flags_hash == 0x0123456789ABCDEF
    assert c.key() == sn.SnapshotKey("naca:4412", 13, 0.08, tuple(g["fcs_dims"]), 1)
    for a, b in zip(c.fields(), g["fcs_fields"]):
        assert np.array_equal(a, b)
    sc = c.scaling()
    for name, val in mg.SNAPSHOT_SCALING.items():
        assert getattr(sc, name) == (val if isinstance(val, int) else np.float32(val)), name
    out = tmp_path / "ours.fcs"
    c.save(out)
    assert out.read_bytes() == src.read_bytes()


@pytest.mark.parametrize("case", range(4))
def test_fcs1_rejections_match_reference(sn, golden, mg, tmp_path, case):
    g = golden("snapshot")
    raw = g["fcs"].tobytes()
    dims = tuple(int(v) for v in g["fcs_dims"])
    bad = [b"XCS1" + raw[4:], raw[:4] + b"\x02" + raw[5:], raw[: len(raw) - 7],
           mg.fcs_bytes(("naca:4412", 13, 0.08, dims, 2), 0x0123456789ABCDEF, mg.SNAPSHOT_SCALING,
                        list(g["fcs_fields"]))][case]
    p = tmp_path / "bad.fcs"
    p.write_bytes(bad)
    c = sn.CompactSnapshot()
    with pytest.raises(Exception) as e:
        c.load(p)
    assert str(e.value).split(":")[0] == str(g["reject_reason"][case])
    assert not c.has_data
    # A payload count that disagrees with the key's grid is refused too.
    big = bytearray(raw)
    off = raw.index((int(np.prod(dims))).to_bytes(8, "little"), 60)
    big[off:off + 8] = (int(np.prod(dims)) + 1).to_bytes(8, "little")
    p.write_bytes(bytes(big))
    with pytest.raises(Exception, match="payload size mismatch"):
        c.load(p)


def _snap(sn, mg, tmp_path, gid, dims=(12, 7, 5), seed=0):
    rng = np.random.default_rng(seed)
    n = int(np.prod(dims))
    fields = [rng.standard_normal(n).astype(np.float32) for _ in range(4)]
    p = tmp_path / f"src_{gid.replace(':', '_')}.fcs"
    p.write_bytes(mg.fcs_bytes((gid, 4, 0.08, dims, 1), 7, mg.SNAPSHOT_SCALING, fields))
    c = sn.CompactSnapshot()
    c.load(p)
    return c


def test_disk_cache_lru_budget_and_hits(sn, mg, tmp_path):
    d = tmp_path / "cache"
    snaps = [_snap(sn, mg, tmp_path, f"naca:00{10 + i}", seed=i) for i in range(4)]
    size = len(mg.fcs_bytes(("naca:0010", 4, 0.08, (12, 7, 5), 1), 7, mg.SNAPSHOT_SCALING,
                            [np.zeros(420, np.float32)] * 4))
    cache = sn.DiskSnapshotCache(d, budget_bytes=3 * size)
    base = time.time() - 1000
    for i, s in enumerate(snaps[:3]):
        cache.store(s)
        path = cache.find(s.key())
        assert path and path.endswith(f"{s.key().hash():016x}.fcs")
        os.utime(path, (base + 10 * i, base + 10 * i))   # distinct, ordered recency
    assert cache.used_bytes == 3 * size
    assert not any(p.suffix == ".tmp" for p in d.iterdir())
    # A hit on the oldest entry refreshes it; the next store evicts the
    # least recently used one (entry 1), never the entry just stored.
    assert cache.find(snaps[0].key())
    cache.store(snaps[3])
    assert cache.find(snaps[1].key()) is None
    for i in (0, 2, 3):
        assert cache.find(snaps[i].key()), i
    assert cache.used_bytes == 3 * size
    # The stored file loads back to the same state.
    c = sn.CompactSnapshot()
    c.load(cache.find(snaps[3].key()))
    for a, b in zip(c.fields(), snaps[3].fields()):
        assert np.array_equal(a, b)
    # A smaller budget evicts at once, oldest first, nothing protected.
    cache.set_budget(size)
    assert cache.used_bytes == size and len(list(d.glob("*.fcs"))) == 1
    cache.close()
    # Reopening scans the directory.
    again = sn.DiskSnapshotCache(d, budget_bytes=10 * size)
    assert again.used_bytes == size
    # A single entry over budget is kept (the store wins).
    again.set_budget(1)
    big = _snap(sn, mg, tmp_path, "naca:9999", seed=9)
    again.store(big)
    assert again.find(big.key()) and again.used_bytes == size
    again.close()


def test_disk_cache_background_writer(sn, mg, tmp_path):
    cache = sn.DiskSnapshotCache(tmp_path / "bg", budget_bytes=1 << 30)
    keys = []
    for i in range(5):
        s = _snap(sn, mg, tmp_path, f"dat:wing{i}.dat", seed=20 + i)
        keys.append(s.key())
        cache.store_async(s)
        assert not s.has_data   # handed over
    cache.wait()
    for k in keys:
        assert cache.find(k)
    cache.close()
