"""Output rows of the library: the VTI writer (the reference's io/vtiWriter.cuh format, byte for
byte, plus raw appended binary), the asynchronous writer that overlaps output with stepping, and
the checkpoint / restart format (a restored case continues bit for bit)."""
import os

import numpy as np
import pytest

import mbcg
from gpu_util import load_fixture

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
ALL_FIELDS = (1 << 11) - 1


def test_vti_ascii_is_byte_identical_to_the_reference_writer(tmp_path):
    p, z = load_fixture("ref_vti_state")
    state = z["state"]
    with mbcg.Case(p) as c:
        c.copy_in(state)
        np.testing.assert_array_equal(c.copy_out(), state)  # the fixture's ghost frame is consistent
        out = tmp_path / "a.vti"
        c.write_vti(str(out))
    assert out.read_bytes() == open(os.path.join(GOLD, "ref_vti_ascii.vti"), "rb").read()


@pytest.mark.parametrize("prec", [mbcg.FP32, mbcg.FP16])
def test_vti_raw_and_ascii_hold_the_state(tmp_path, prec):
    p = mbcg.jet_params(40, 36, 30, q=27, diameter=10.0, precision=prec)
    with mbcg.Case(p) as c:
        c.init()
        c.step(7)
        ref = c.copy_out()
        c.write_vti(str(tmp_path / "r.vti"), fields=ALL_FIELDS, fmt=mbcg.VTI_RAW)
        c.write_vti(str(tmp_path / "a.vti"), fields=0b101, fmt=mbcg.VTI_ASCII)
    raw = mbcg.read_vti(str(tmp_path / "r.vti"))
    assert list(raw) == list(mbcg.FIELD_NAMES)
    for f, name in enumerate(mbcg.FIELD_NAMES):
        np.testing.assert_array_equal(raw[name], ref[f])
    asc = mbcg.read_vti(str(tmp_path / "a.vti"))  # %.8e keeps every float32 exactly
    assert list(asc) == ["rhor", "ux"]
    np.testing.assert_array_equal(asc["rhor"], ref[0])
    np.testing.assert_array_equal(asc["ux"], ref[2])


def test_async_writer_matches_synchronous_states(tmp_path):
    p = mbcg.jet_params(40, 36, 50, q=19, diameter=10.0)
    marks = (3, 8, 9, 15)
    expected = {}
    with mbcg.Case(p) as c:
        c.init()
        done = 0
        for m in marks:
            c.step(m - done)
            done = m
            expected[m] = c.copy_out()
    with mbcg.Case(p) as c, mbcg.Writer(max_pending=2) as w:
        c.init()
        done = 0
        for m in marks:
            c.step(m - done)  # enqueued; the snapshot below is ordered after it on the same stream
            done = m
            w.snapshot(c, str(tmp_path / f"s{m}.vti"), fields=ALL_FIELDS, fmt=mbcg.VTI_RAW)
        c.step(5)  # keeps stepping while the files are written
        w.flush()
    for m in marks:
        got = mbcg.read_vti(str(tmp_path / f"s{m}.vti"))
        for f, name in enumerate(mbcg.FIELD_NAMES):
            np.testing.assert_array_equal(got[name], expected[m][f], err_msg=f"step {m} {name}")


CKPT_CASES = {
    "jet_fp32": lambda: mbcg.jet_params(40, 36, 30, q=27, diameter=10.0),  # seeded inlet noise: the counter matters
    "rti_fp16": lambda: mbcg.rti_params(24, 40, q=19, precision=mbcg.FP16),
    "bubble_bf16": lambda: mbcg.bubble_params(30, q=27, radius=8.0, precision=mbcg.BF16),
}


@pytest.mark.parametrize("name", sorted(CKPT_CASES))
def test_checkpoint_restart_is_bit_exact(tmp_path, name):
    p = CKPT_CASES[name]()
    path = str(tmp_path / "c.mbcg")
    with mbcg.Case(p) as c:
        c.init()
        c.step(7)
        c.checkpoint(path)
        c.step(9)
        ref = c.copy_out()
    with mbcg.Case.from_checkpoint(path) as r:
        assert r.steps_done == 7
        assert r.params.describe() == p.describe()
        r.step(9)
        np.testing.assert_array_equal(r.copy_out(), ref)


def test_checkpoint_rejects_damaged_files(tmp_path):
    p = mbcg.bubble_params(20, q=19)
    path = tmp_path / "c.mbcg"
    with mbcg.Case(p) as c:
        c.init()
        c.checkpoint(str(path))
    good = path.read_bytes()
    flipped = bytearray(good)
    flipped[-100] ^= 0x40
    bad = tmp_path / "bad.mbcg"
    for data in (bytes(flipped), good[:-1000], b"NOTMBCG!" + good[8:]):
        bad.write_bytes(data)
        with pytest.raises(mbcg.MbcgError):
            mbcg.Case.from_checkpoint(str(bad))
