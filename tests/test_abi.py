"""The C ABI library loads without a GPU, exports every declared symbol, and its
planner follows the reference's admission rules."""
import re
from pathlib import Path

import numpy as np
import pytest

import nttanafis_gb300 as ntt

ROOT = Path(__file__).resolve().parents[1]
MASK = (1 << 64) - 1


def declared_symbols(header: str = "ntt_gb300.h"):
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ntt_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = ntt.library()
    names = declared_symbols()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert sorted(ntt.exported_symbols()) == names


def test_probe_library_is_separate_and_exports_its_header():
    from nttanafis_gb300 import probe

    lib = probe.library()
    names = declared_symbols("ntt_probe.h")
    for name in names:
        assert hasattr(lib, name), name
    assert sorted(probe.exported_symbols()) == names
    assert not set(names) & set(declared_symbols())  # nothing of it in the product ABI
    assert lib.ntt_probe_variants() == len(probe.VARIANTS)


def test_version_and_counters():
    assert b"sm_103a" in ntt.library().ntt_version()
    assert ntt.kernel_launches() >= 0


def test_mul_plans_reject_like_the_reference(golden):
    for la, lb in golden["rejections"]["mul_none"]:
        assert ntt.MulPlan.new(la, lb) is None
    for la, lb in [(1, 1), (3, 7), (4, 4), (16, 65), (257, 256)]:
        p = ntt.MulPlan.new(la, lb)
        assert p is not None and p.scratch_len() >= p.sqr_scratch_len()
    # beyond one 2^25-point transform: admitted through the block split while the
    # shorter operand fits a block transform, rejected otherwise
    p = ntt.MulPlan.new(2**25, 2)
    assert p is not None and p.blocks > 1
    assert ntt.MulPlan.new(2**25, 2**25) is None
    assert ntt.MulPlan.new(2**41, 8) is None


def test_conv_strides_match_reference_table(golden):
    for terms, ma, mb, stride in golden["strides"]["cases"]:
        assert ntt.ConvPlan.new(terms, terms, ma, mb, False).stride() == stride


def test_conv_plans_reject_like_the_reference(golden):
    for la, lb, ma, mb, s in golden["rejections"]["conv_none"]:
        assert ntt.ConvPlan.new(la, lb, ma, mb, bool(s)) is None
    p = ntt.ConvPlan.new(3, 2, 3, 5, False)
    # the reference's schoolbook plans need no scratch for their arithmetic
    # (src/convolve.rs:132); the device call's scratch holds only the 512 bytes of
    # the on-device admission votes, in front of the residues of transform plans
    assert p.output_len() == 4 and p.schoolbook and p.scratch_len() == 64
    big = ntt.ConvPlan.new(30, 30, 7, 7, False)
    assert big.scratch_len() > 64 and not big.schoolbook


def test_conv_plan_matches_oracle_stride_and_output():
    import oracle

    rng = np.random.default_rng(3)
    for _ in range(200):
        la, lb = int(rng.integers(1, 5000)), int(rng.integers(1, 5000))
        bits_a, bits_b = int(rng.integers(0, 65)), int(rng.integers(0, 65))
        signed = bool(rng.integers(0, 2))
        ma = (1 << bits_a) - 1 if bits_a < 64 else MASK
        mb = (1 << bits_b) - 1 if bits_b < 64 else MASK
        if signed:
            ma, mb = min(ma, (1 << 63) - 1), min(mb, (1 << 63) - 1)
        ours = ntt.ConvPlan.new(la, lb, ma, mb, signed)
        ref = oracle.conv_plan(la, lb, ma, mb, signed)
        assert (ours is None) == (ref is None)
        if ours is not None:
            assert ours.stride() == ref["stride"] and ours.output_len() == ref["output_len"]
            assert ours.schoolbook == bool(ref["schoolbook"])


def test_plans_hold_every_coefficient():
    # the transform holds the whole product, or one block times the shorter operand
    for la, lb in [(1, 1), (1024, 1024), (2**20, 2**20), (2**20, 131072), (2**24, 2**24), (2**25 - 5, 5),
                   (65536, 256), (3000, 1), (2**30, 1000)]:
        p = ntt.MulPlan.new(la, lb)
        assert p is not None, (la, lb)
        if p.blocks:
            assert (1 << p.log_transform) >= p.block_len + min(la, lb) - 1
            assert p.block_len >= min(la, lb)  # blocks of one parity never overlap
            assert p.blocks * p.block_len >= max(la, lb) > (p.blocks - 1) * p.block_len
        else:
            assert (1 << p.log_transform) >= la + lb - 1


def test_fewest_primes_per_length():
    # five primes hold every product: lazy ones up to 2^21 points and where they
    # suffice at 2^22 (148 bits) and 2^23 (147); wide ones beyond, and at 2^22, 2^23
    # where five lazy primes fall a bit short (six would be needed)
    for la, lb in [(1024, 1024), (2**20, 2**20), ((1 << 22) - 2**20, 2**20), ((1 << 22) - 2**20 - 1, 2**20 + 1),
                   ((1 << 23) - 2**19, 2**19), ((1 << 23) - 2**19 - 1, 2**19 + 1), (2**22, 2**22), (2**24, 2**24)]:
        p = ntt.MulPlan.new(la, lb)
        assert p.primes == 5 and p.blocks == 0, (la, lb)
        assert p.log_transform == max(4, (la + lb - 2).bit_length()), (la, lb)
    # convolutions: 16-bit and 32-bit classes unchanged, 64-bit coefficients over
    # 2^20 terms at 2^22 points on five primes (149 bits)
    assert ntt.ConvPlan.new(2**22, 2**22, 0xFFFF, 0xFFFF, False).primes == 2
    assert ntt.ConvPlan.new(2**22, 2**22, 2**32 - 1, 2**32 - 1, False).primes == 3
    wide = ntt.ConvPlan.new(3 * 2**20 - 7, 2**20 + 3, 2**64 - 1, 2**64 - 1, False)
    assert wide.primes == 5 and wide.log_transform == 22 and wide.stride() == 3


def test_block_split_choice():
    # very unbalanced shapes split; balanced ones and squares never do
    assert ntt.MulPlan.new(2**20, 1024).blocks > 1
    assert ntt.MulPlan.new(1024, 2**20).blocks > 1
    assert ntt.MulPlan.new(2**20, 131072).blocks > 1
    assert ntt.MulPlan.new(2**20, 2**20).blocks == 0
    assert ntt.MulPlan.new(4096, 4096).blocks == 0
    assert ntt.MulPlan.new(300, 40).blocks == 0  # below the smallest block transform
    split = ntt.MulPlan.new(2**20, 1024)
    whole_log = (2**20 + 1024 - 1 - 1).bit_length()
    assert split.log_transform < whole_log


def test_split_api_ranges_and_validation():
    # four-step splits: columns 2^6..2^11, rows 2^7..2^13, lazy lengths 2^14..2^23
    assert ntt.split_range(13) is None and ntt.split_range(24) is None
    assert ntt.split_range(14) == (6, 7)
    assert ntt.split_range(21) == (8, 11)
    assert ntt.split_range(23) == (10, 11)
    assert ntt.get_split(21) == 10 and ntt.get_split(13) == 0
    with pytest.raises(ValueError):
        ntt.set_split(21, 12)
    with pytest.raises(ValueError):
        ntt.set_split(21, 7)
    with pytest.raises(ValueError):
        ntt.set_split(20, 6)
    with pytest.raises(ValueError):
        ntt.set_split(13, 6)
    try:
        assert ntt.set_split(21, 9) == 10
        assert ntt.get_split(21) == 9
    finally:
        assert ntt.set_split(21, 0) == 9
    assert ntt.get_split(21) == 10


def test_split_file_round_trip(tmp_path):
    try:
        ntt.set_split(18, 10)
        path = tmp_path / "splits.json"
        ntt.save_splits(path)
        ntt.set_split(18, 0)
        assert ntt.load_splits(path)[18] == 10
        assert ntt.get_split(18) == 10
    finally:
        ntt.set_split(18, 0)


def test_repeated_plans_are_identical_and_failures_repeat():
    # plans are cached per thread: a repeated shape returns the same plan, and a
    # rejected shape is rejected again with its message
    shapes = [(1000, 900), (1 << 20, 1 << 20), (65536, 256), (2**25, 2), (7, 5)]
    first = [ntt.MulPlan.new(a, b) for a, b in shapes]
    again = [ntt.MulPlan.new(a, b) for a, b in shapes]
    assert first == again
    for _ in range(2):
        assert ntt.MulPlan.new(2**25, 2**25) is None
        assert ntt.last_error()
    c1 = ntt.ConvPlan.new(3000, 2000, 0xFFFF, 0xFFFF, False)
    c2 = ntt.ConvPlan.new(3000, 2000, 0xFFFF, 0xFFFF, False)
    assert c1 == c2 and c1 is not None
    assert ntt.ConvPlan.new(3000, 2000, 0xFFFF, 0xFFFF, True) != c1
