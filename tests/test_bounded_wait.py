"""k_scatter's bounded waits: when a wait runs out, the block stops issuing copies, waits for
the ones in flight, skips its remaining work and sets an error bit; the host reports GZ_TIMEOUT
at the next synchronising call and the device stays usable.

The waits are made to run out by lowering their poll limit to one poll (gz_debug_set_spin_limit):
the copy-issuing warp of every tile then gives up on its first wait for a free staging slot,
which the scattering warps release only after sorting the tile.  No wait is left without a
limit, and nothing faults."""
import numpy as np
import pytest

from gazelle_plugin_gb300 import shuffle as S
from gazelle_plugin_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _split(batches, spin_limit=None):
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", W.C2_PARTITIONS, None, W.C2_KEYS, list(W.C2_SCHEMA)),
               writeSchema=False)
    try:
        if spin_limit is not None:
            w.setSpinLimit(h, spin_limit)
        for b in batches:
            a, z = b.addrs_sizes()
            w.split(h, b.num_rows, a, z)
        w.stop(h, W.C2_PARTITIONS)
        return w.data(h)
    finally:
        w.close(h)


def test_wait_that_runs_out_reports_timeout_and_device_stays_usable():
    batches = W.c2_batches(51, 6, 4096)
    with pytest.raises(S.SplitterError) as ei:
        _split(batches, spin_limit=1)
    assert ei.value.status == S.GZ_TIMEOUT
    # the same batches again with the default limit: complete and equal to the oracle
    got = _split(batches)
    ref = O.run_oracle(W.C2_SCHEMA, batches, W.C2_PARTITIONS, W.C2_KEYS)
    assert got == ref.data
