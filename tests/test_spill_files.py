"""Partition data past host_budget goes to local-dir files (the reference spills cached record
batches to temp_shuffle_* files in <local dir>/<2-hex-digit sub dir>, splitter.cc:75-82, 120,
1346-1353; utils.h:55-115) and is read back at Stop: the data file's bytes do not change."""
import numpy as np
import pytest

from gazelle_plugin_gb300 import workloads as W
from oracle import ipc_read as R
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _split_with_files(tmp_path, batches, codec=None):
    from gazelle_plugin_gb300 import shuffle as S
    dirs = [tmp_path / "d0", tmp_path / "d1"]
    w = S.ShuffleSplitterJniWrapper()
    kw = {"codec": codec} if codec else {}
    h = w.make(S.NativePartitioning("hash", 200, None, W.C2_KEYS, list(W.C2_SCHEMA)), writeSchema=False,
               localDirs=",".join(str(d) for d in dirs), subDirsPerLocalDir=4, keep_output_on_device=0,
               flush_bytes=1 << 20, host_budget=2 << 20, **kw)
    for b in batches:
        a, z = b.addrs_sizes()
        w.split(h, b.num_rows, a, z)
    w.sync(h)
    files, nbytes, now = w.diskSpill(h)
    assert files >= 3 and now == files and nbytes > 0
    on_disk = sorted(tmp_path.rglob("temp_shuffle_*"))
    assert len(on_disk) == now
    assert {p.parent.parent for p in on_disk} == set(dirs)  # both dirs, in turn
    assert all(len(p.parent.name) == 2 and int(p.parent.name, 16) < 4 for p in on_disk)
    assert sum(p.stat().st_size for p in on_disk) == nbytes
    res = w.stop(h)
    data = w.data(h)
    assert w.diskSpill(h)[2] == 0 and not list(tmp_path.rglob("temp_shuffle_*"))
    w.close(h)
    return res, data


def test_passes_spilled_to_local_dir_files_read_back_at_stop(tmp_path):
    batches = W.c2_batches(81, 40, 4096)
    res, data = _split_with_files(tmp_path, batches)
    ref = O.run_oracle(W.C2_SCHEMA, batches, 200, W.C2_KEYS)
    assert data == ref.data
    assert np.array_equal(res.partitionLengths, ref.partition_lengths)
    assert np.array_equal(res.rawPartitionLengths, ref.raw_partition_lengths)


def test_lz4_output_with_passes_in_local_dir_files(tmp_path):
    from gazelle_plugin_gb300 import shuffle as S
    batches = W.c2_batches(82, 24, 4096)
    res_z, data_z = _split_with_files(tmp_path, batches, codec="lz4")
    res_u, data_u = S.split_batches(W.C2_SCHEMA, batches, 200, W.C2_KEYS, writeSchema=False)
    st_u = np.concatenate([[0], np.cumsum(np.asarray(res_u.partitionLengths))])
    st_z = np.concatenate([[0], np.cumsum(np.asarray(res_z.partitionLengths))])
    for p in range(200):
        bu = R.parse_stream(data_u[st_u[p]:st_u[p + 1]], W.C2_SCHEMA)
        bz = R.parse_stream(data_z[st_z[p]:st_z[p + 1]], W.C2_SCHEMA)
        assert [r for r, _ in bu] == [r for r, _ in bz]
        for (_, cu), (_, cz) in zip(bu, bz):
            assert [[bytes(x) for x in f[1]] for f in cu] == [[bytes(x) for x in f[1]] for f in cz]


def test_host_budget_needs_local_dirs():
    from gazelle_plugin_gb300 import shuffle as S
    w = S.ShuffleSplitterJniWrapper()
    with pytest.raises(S.SplitterError) as e:
        w.make(S.NativePartitioning("hash", 8, None, W.C1_KEYS, list(W.C1_SCHEMA)), writeSchema=False,
               host_budget=1 << 20)
    assert e.value.status == S.GZ_INVALID
