"""Weight snapshot files in the reference's NPGR_WEIGHT_SNAPSHOT v1 format
(src/native/gpu/src/simulation_dense/SimulationWeightIO.cpp): exact-equality
run-length encoding, 9 significant digits (every float32 survives the round
trip bit for bit), and the reader's structural checks with the reference's
reason texts."""
import numpy as np
import pytest

from neuronbridge_gb300.weightio import read_snapshot, write_snapshot


def test_layout_of_a_small_snapshot(tmp_path):
    p = tmp_path / "w.dat"
    write_snapshot(p, np.array([0.5, 0.5, 0.5, 0.25, 1.0 / 3.0], np.float32), 41,
                   dense_blocks=[('motor "a"', np.array([2.0, 2.0], np.float32))])
    assert p.read_text() == (
        "NPGR_WEIGHT_SNAPSHOT 1\ntime_step 41\n\n"
        "block main 0 5\nrle\n3 0.5\n1 0.25\n1 0.333333343\nend_block\n\n"
        'block dense 0 "motor \\"a\\"" 2\nrle\n2 2\nend_block\n\n'
        "end\n")
    snap = read_snapshot(p)
    assert snap["time_step"] == 41
    assert snap["dense"][0][:2] == (0, 'motor "a"')
    assert np.array_equal(snap["dense"][0][2], [2.0, 2.0])


def test_round_trip_is_bit_exact(tmp_path):
    rng = np.random.default_rng(3)
    w = rng.standard_normal(20000).astype(np.float32)
    w[100:400] = 0.0                       # long runs
    w[5000:5003] = np.float32(1e-38)       # subnormal-adjacent values
    w[7] = np.float32(-0.0)
    p = tmp_path / "w.dat"
    write_snapshot(p, w, 0)
    got = read_snapshot(p)["main"]
    assert got.dtype == np.float32 and np.array_equal(got.view(np.uint32)[w != 0], w.view(np.uint32)[w != 0])
    assert np.array_equal(got, w)


def test_empty_main_block(tmp_path):
    p = tmp_path / "w.dat"
    write_snapshot(p, np.zeros(0, np.float32), 3)
    assert len(read_snapshot(p)["main"]) == 0


@pytest.mark.parametrize("text,reason", [
    ("WEIGHTS 1\n", "not an NPGR_WEIGHT_SNAPSHOT v1 file"),
    ("NPGR_WEIGHT_SNAPSHOT 2\ntime_step 0\nend\n", "not an NPGR_WEIGHT_SNAPSHOT v1 file"),
    ("NPGR_WEIGHT_SNAPSHOT 1\nstep 0\nend\n", "missing time_step"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nend\n", "missing main block"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nblock main 1 0\nrle\nend_block\nend\n", "main weight block header is invalid"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nblock main 0 2\nraw\n", "missing rle marker"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nblock main 0 2\nrle\n0 1.0\nend_block\nend\n", "non-positive run count"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nblock main 0 2\nrle\n3 1.0\nend_block\nend\n", "expands beyond"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nblock main 0 2\nrle\n1 1.0\nend_block\nend\n", "unexpected weight count"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nblock main 0 2\nrle\nx 1.0\nend_block\nend\n", "invalid run count"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nblock main 0 2\nrle\n2\n", "missing a weight value"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nblock main 0 2\nrle\n2 1.0\n", "end-of-file before end_block"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nblock main 0 0\nrle\nend_block\n"
     "block main 0 0\nrle\nend_block\nend\n", "duplicate main blocks"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nblock sparse 0 0\nend\n", "unknown block kind"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nweights\nend\n", "unexpected token"),
    ("NPGR_WEIGHT_SNAPSHOT 1\ntime_step 0\nblock main 0 0\nrle\nend_block\n", "end-of-file before end marker"),
])
def test_reader_rejects_malformed_files(tmp_path, text, reason):
    p = tmp_path / "bad.dat"
    p.write_text(text)
    with pytest.raises(ValueError, match=reason):
        read_snapshot(p)


def test_missing_file(tmp_path):
    with pytest.raises(ValueError, match="failed to open weight snapshot for reading"):
        read_snapshot(tmp_path / "absent.dat")
