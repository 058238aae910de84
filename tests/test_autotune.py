"""The autotuner (gz_autotune, gz_tune_save / gz_tune_load): pass size and segment length chosen
by measurement per schema signature.  The cache file round-trips on the CPU; on the GPU a tuned
splitter (flush_bytes=0, seg_tiles=0) must give exactly the bytes of the default one, whatever
settings were chosen."""
import os

import numpy as np
import pytest

from gazelle_plugin_gb300 import shuffle as S
from gazelle_plugin_gb300 import workloads as W
from oracle import oracle as O


def test_cache_file_round_trip(tmp_path):
    src = tmp_path / "in.txt"
    src.write_text("t=4,5;k=0;P=8 16777216 4 12.500\n"
                   "not a valid line\n"
                   "t=4,9,13;k=0,1;P=200 67108864 0 40.250\n")
    S.tune_load(str(src))
    out = tmp_path / "out.txt"
    S.tune_save(str(out))
    lines = out.read_text().splitlines()
    assert "t=4,5;k=0;P=8 16777216 4 12.500" in lines
    assert "t=4,9,13;k=0,1;P=200 67108864 0 40.250" in lines
    assert not any("valid" in l for l in lines)


def test_missing_cache_file_is_an_io_error(tmp_path):
    with pytest.raises(S.SplitterError) as e:
        S.tune_load(str(tmp_path / "absent.txt"))
    assert e.value.status == S.GZ_IO


@pytest.mark.gpu
@pytest.mark.parametrize("si", [0, 1, 2])
def test_tuned_splitter_gives_the_default_bytes(si):
    rng = np.random.Generator(np.random.PCG64(40 + si))
    schema, keys = W.C4_SCHEMAS[si]
    P = W.C4_PARTITIONS[si]
    batches = [W.c4_batch(rng, si, int(r)) for r in W.c4_rows(rng, 24)]
    r = S.autotune(schema, P, keys, batches, writeSchema=False)
    assert r["runs"] >= 2 and r["best_gbs"] > 0 and r["default_gbs"] > 0
    assert (16 << 20) <= r["flush_bytes"] <= (1 << 30) and 0 <= r["seg_tiles"] <= 32
    tuned, tdata = S.split_batches(schema, batches, P, keys, writeSchema=False, flush_bytes=0, seg_tiles=0)
    ref, rdata = S.split_batches(schema, batches, P, keys, writeSchema=False)
    assert tdata == rdata
    assert np.array_equal(tuned.partitionLengths, ref.partitionLengths)
    oracle = O.run_oracle(schema, batches, P, keys, buffer_size=4096)
    assert rdata == oracle.data


@pytest.mark.gpu
def test_every_segment_length_gives_the_same_bytes():
    rng = np.random.Generator(np.random.PCG64(44))
    schema, keys = W.C4_SCHEMAS[1]
    batches = [W.c4_batch(rng, 1, int(r)) for r in W.c4_rows(rng, 12)]
    ref, rdata = S.split_batches(schema, batches, 200, keys, writeSchema=False)
    for seg in (1, 2, 4, 8, 16, 32):
        for flush in (1 << 20, 64 << 20):
            res, data = S.split_batches(schema, batches, 200, keys, writeSchema=False,
                                        flush_bytes=flush, seg_tiles=seg)
            assert data == rdata, (seg, flush)
            assert np.array_equal(res.partitionLengths, ref.partitionLengths)
