"""The packed host layout of a batch (the arrays ilm_batch_create,
ilm_batch_set_learned and ilm_batch_set_coarse read) built from problem
specs: records byte-identical to the C struct, points concatenated in
problem order, body starts local to each problem."""
import ctypes as C

import numpy as np


def test_packed_batch_layout():
    from immersedlayers import _lib as L
    from immersedlayers import workloads as W
    from immersedlayers.batch import PackedBatch
    specs = W.batch_specs(12)
    pk = PackedBatch(specs)
    # records: the same bytes as an array of the C struct
    arr = (L.BatchProblem * len(specs))()
    for i, s in enumerate(specs):
        arr[i] = L.BatchProblem(s.nx, s.ny, s.h, s.i0[0], s.i0[1], s.npts, s.kind)
    assert pk.records.itemsize == C.sizeof(L.BatchProblem)
    assert bytes(arr) == pk.records.tobytes()
    # points: problem order, body order within a problem
    for a, got in zip(("x", "y", "nx", "ny", "ds"), pk.points):
        want = np.concatenate([getattr(s.bl, a) for s in specs])
        assert got.dtype == np.float64 and got.flags["C_CONTIGUOUS"]
        assert np.array_equal(got, want)
    # body starts: local index of the first point of each point's body
    off = 0
    for s in specs:
        fi = s.bl.firstindices()
        for b in range(len(fi) - 1):
            assert (pk.body_starts[off + fi[b]:off + fi[b + 1]] == fi[b]).all()
        off += s.npts
    assert off == pk.body_starts.size and pk.body_starts.dtype == np.int32
    assert pk.nbytes == pk.records.nbytes + 5 * 8 * off
