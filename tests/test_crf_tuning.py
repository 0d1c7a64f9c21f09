"""CPU tests of the CRF tile table (cnncrf_crf_tuning_*): set / get / count /
clear, the argument checks, and the text file: save, merge on load, and a
malformed file that is rejected with the table left unchanged.  No GPU: the
table is host state."""
import pytest


@pytest.fixture()
def tuning():
    from cnncrf import tuning as T
    T.clear()
    yield T
    T.clear()


def test_default_and_set_get(tuning):
    tile, found, mh, mv = tuning.get_tile(1242, 375, 128, 4, 3)
    assert not found and tile == tuning.DEFAULT and mh == mv == 0.0
    tuning.set_tile(1242, 375, 128, 4, 3, ring_h=4, chains_per_cta_h=1, chains_per_cta_v=4)
    tile, found, _, _ = tuning.get_tile(1242, 375, 128, 4, 3)
    assert found and tile == dict(ring_h=4, chains_per_cta_h=1, ring_v=8, chains_per_cta_v=4)
    # the key is the whole shape: another pair count or delta is another entry
    assert not tuning.get_tile(1242, 375, 128, 8, 3)[1]
    assert not tuning.get_tile(1242, 375, 128, 4, 2)[1]
    assert tuning.count() == 1
    tuning.clear()
    assert tuning.count() == 0


@pytest.mark.parametrize("bad", [dict(ring_h=6), dict(ring_v=16), dict(chains_per_cta_h=3),
                                 dict(chains_per_cta_v=0)])
def test_invalid_tiles_rejected(tuning, bad):
    from cnncrf import _lib as L
    with pytest.raises(L.CnnCrfError) as e:
        tuning.set_tile(64, 32, 16, 1, 2, **bad)
    assert e.value.status == L.EINVAL
    assert tuning.count() == 0


@pytest.mark.parametrize("shape", [(0, 32, 16, 1, 2), (64, 32, 257, 1, 2), (64, 32, 16, 0, 2), (64, 32, 16, 1, 5)])
def test_invalid_shapes_rejected(tuning, shape):
    from cnncrf import _lib as L
    with pytest.raises(L.CnnCrfError) as e:
        tuning.set_tile(*shape)
    assert e.value.status == L.EINVAL


def test_save_load_round_trip_and_merge(tuning, tmp_path):
    tuning.set_tile(480, 320, 64, 4, 3, ring_h=4, ring_v=4)
    tuning.set_tile(1440, 960, 192, 4, 3, ring_h=4, chains_per_cta_h=4, chains_per_cta_v=4)
    f = tmp_path / "tiles.txt"
    tuning.save(f)
    text = f.read_text().splitlines()
    assert text[0] == "cnncrf-crf-tiles 1" and text[1].startswith("#") and len(text) == 4
    tuning.clear()
    tuning.set_tile(720, 480, 96, 4, 3, chains_per_cta_h=1)  # kept: load merges
    tuning.load(f)
    assert tuning.count() == 3
    assert tuning.get_tile(1440, 960, 192, 4, 3)[0] == dict(ring_h=4, chains_per_cta_h=4, ring_v=8,
                                                            chains_per_cta_v=4)
    assert tuning.get_tile(720, 480, 96, 4, 3)[0]["chains_per_cta_h"] == 1


@pytest.mark.parametrize("body", [
    "not-a-tile-file\n",
    "cnncrf-crf-tiles 1\n64 32 16 1 2 8 2 8 2 0.1 0.1\n64 32 16 1 2 6 2 8 2 0.1 0.1\n",  # ring 6
    "cnncrf-crf-tiles 1\n64 32 16 1 2 8 2 8\n",                                         # short line
    "cnncrf-crf-tiles 1\n64 32 16 1 2 8 2 8 2 0.1 0.1 extra\n",                          # trailing field
    "",
])
def test_malformed_file_changes_nothing(tuning, tmp_path, body):
    from cnncrf import _lib as L
    tuning.set_tile(100, 50, 32, 2, 2, ring_v=4)
    f = tmp_path / "bad.txt"
    f.write_text(body)
    with pytest.raises(L.CnnCrfError) as e:
        tuning.load(f)
    assert e.value.status == L.EINVAL
    assert tuning.count() == 1 and tuning.get_tile(100, 50, 32, 2, 2)[0]["ring_v"] == 4
    assert not tuning.get_tile(64, 32, 16, 1, 2)[1]


def test_comments_and_blank_lines(tuning, tmp_path):
    f = tmp_path / "c.txt"
    f.write_text("cnncrf-crf-tiles 1\n\n# a comment\n   # indented comment\n64 32 16 1 2 4 1 8 4 0.5 0.25\n")
    tuning.load(f)
    tile, found, mh, mv = tuning.get_tile(64, 32, 16, 1, 2)
    assert found and tile == dict(ring_h=4, chains_per_cta_h=1, ring_v=8, chains_per_cta_v=4)
    assert (mh, mv) == (0.5, 0.25)
