"""Snapshots (gtc_write_snapshot / gtc_read_snapshot): the content of the
reference's GADGET snapshots (src/snapshot_io.cpp:113-221) in a raw binary
file. A round trip keeps every field; particles come back grouped by type in
ascending type order, stable within a type, as the reference's reader
returns them; bad files and mismatched sizes are refused."""

import numpy as np
import pytest


def test_round_trip_groups_by_type(gtc, tmp_path):
    pos, vel, mass, typ = gtc.make_galaxy(3000, seed=2)
    rng = np.random.default_rng(1)
    typ = typ.astype(np.uint8)
    typ[::7] = 5
    ids = rng.permutation(10_000)[:3000].astype(np.uint64)
    pot = rng.normal(size=3000)
    path = tmp_path / "snap.gtsnap"
    gtc.write_snapshot(path, pos, vel, mass, ids=ids, types=typ, pot=pot, time=1.25,
                       metadata={"gravity": "group", "theta": "0.75"})
    s = gtc.read_snapshot(path)
    order = np.argsort(typ, kind="stable")
    assert s["time"] == 1.25
    assert s["count_by_type"].tolist() == [int((typ == t).sum()) for t in range(6)]
    for key, want in (("pos", pos), ("vel", vel), ("mass", mass), ("ids", ids), ("types", typ),
                      ("pot", pot)):
        assert np.array_equal(s[key], want[order]), key
    assert s["metadata"] == {"gravity": "group", "theta": "0.75"}


def test_defaults_and_empty(gtc, tmp_path):
    pos = np.arange(12.0).reshape(4, 3)
    path = tmp_path / "a.gtsnap"
    gtc.write_snapshot(path, pos, -pos, np.ones(4))
    s = gtc.read_snapshot(path)
    assert s["types"].tolist() == [1, 1, 1, 1] and s["ids"].tolist() == [0, 1, 2, 3]
    assert np.all(s["pot"] == 0) and s["metadata"] == {}
    gtc.write_snapshot(tmp_path / "e.gtsnap", np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0))
    assert gtc.read_snapshot(tmp_path / "e.gtsnap")["mass"].shape == (0,)


def test_refuses_bad_files(gtc, tmp_path):
    with pytest.raises(gtc.GtcError):
        gtc.read_snapshot(tmp_path / "missing.gtsnap")
    bad = tmp_path / "bad.gtsnap"
    bad.write_bytes(b"not a snapshot at all, just some bytes for the header..........")
    with pytest.raises(gtc.GtcError) as e:
        gtc.read_snapshot(bad)
    assert "GTSNAP01" in str(e.value)
    good = tmp_path / "g.gtsnap"
    gtc.write_snapshot(good, np.zeros((5, 3)), np.zeros((5, 3)), np.ones(5))
    cut = tmp_path / "cut.gtsnap"
    cut.write_bytes(good.read_bytes()[:150])
    with pytest.raises(gtc.GtcError) as e:
        gtc.read_snapshot(cut)
    assert "truncated" in str(e.value)
    with pytest.raises(gtc.GtcInvalidArgument):
        gtc.write_snapshot(good, np.zeros((2, 3)), np.zeros((2, 3)), np.ones(2),
                           types=np.array([1, 9], np.uint8))
