"""ufo_track_noalloc: the entry point for callers that cannot allocate.

Some callers cannot call cudaMalloc -- a program whose GPU memory belongs to
another allocator, or an online model that must not allocate while it runs.
ufo_track_noalloc takes every buffer from the caller and keeps its own
scratch (the staged opcode table and the work counter) in a static device
array.  These tests call it through the C ABI with caller-owned device
buffers and compare it with the regular entry point, ufo_track, which
allocates its own buffers; in the default (strict) mode both must agree bit
for bit.  This file is collected last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest


def _noalloc(prog, coords, turns, mode, flags=0):
    import torch
    from ufo_gb300 import capi
    lib = capi.load()
    torch.cuda.set_device(0)
    dev = torch.device('cuda', 0)
    ops = np.ascontiguousarray(prog.ops, dtype=np.int32)
    table = torch.from_numpy(np.ascontiguousarray(prog.table, dtype=np.float64)).to(dev)
    c = torch.from_numpy(np.ascontiguousarray(coords, dtype=np.float64)).to(dev)
    n = coords.shape[0]
    lost = torch.full((n,), -7, dtype=torch.int32, device=dev)
    final = torch.full((n, 6), np.nan, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = lib.ufo_track_noalloc(capi.ptr(ops), ops.shape[0], capi.ptr(table.data_ptr()),
                               table.shape[1], table.shape[0], int(prog.n_dumps),
                               capi.ptr(c.data_ptr()), None, None, n, int(turns), int(mode),
                               int(flags), 0, 1, None, capi.ptr(lost.data_ptr()),
                               capi.ptr(final.data_ptr()), None)
    capi.check(rc)
    torch.cuda.synchronize()
    return lost.cpu().numpy().view(np.uint32), final.cpu().numpy()


@pytest.mark.gpu
def test_noalloc_matches_regular_entry_point_two_calls():
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    ctx = u.context(0)
    # call 1: dynamic-aperture grid (StableAperture mode) on the C1 ring with
    # apertures and multipole errors
    ring = W.c3_ring(u)
    p1 = C.compile_line(ring, u.KICK, where=[-1])
    grid = W.c3_grid(20, 20)
    _, lost_ref, final_ref = capi.track(ctx, capi.DeviceProgram(ctx, p1), grid, 300,
                                        capi.UFO_MODE_SA, 0, slots=0)
    lost, final = _noalloc(p1, grid, 300, capi.UFO_MODE_SA)
    assert np.array_equal(lost, lost_ref)
    assert np.array_equal(final, final_ref, equal_nan=True)
    assert 0 < np.sum(lost < 300) < lost.size
    # call 2, right after: another lattice and mode through the same scratch
    ring2 = W.c2_ring(u)
    p2 = C.compile_line(ring2, u.KICK, where=[-1])
    beam = W.c2_beam(3000, seed=9)
    _, lost_ref2, final_ref2 = capi.track(ctx, capi.DeviceProgram(ctx, p2), beam, 50,
                                          capi.UFO_MODE_TRACK, 0, slots=0)
    lost2, final2 = _noalloc(p2, beam, 50, capi.UFO_MODE_TRACK)
    assert np.array_equal(lost2, lost_ref2)
    assert np.array_equal(final2, final_ref2, equal_nan=True)


def test_noalloc_rejects_oversized_table_before_touching_the_gpu():
    from ufo_gb300 import capi
    lib = capi.load()
    ops = np.zeros((8193, 8), dtype=np.int32)
    table = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    rc = lib.ufo_track_noalloc(capi.ptr(ops), 8193, table, 1, 1, 0, None, None, None, 0, 1, 0,
                               0, 0, 1, None, None, None, None)
    assert rc == -1
    assert b'maximum of 8192' in lib.ufo_last_error()


@pytest.mark.parametrize('index', [-1, 1])
def test_noalloc_rejects_observation_index_outside_dumps_before_touching_the_gpu(index):
    """An observation op writes slot (turn / every) * n_dumps + index of each
    particle's track rows; an index outside [0, n_dumps) would write into
    another particle's rows (or before the buffer), so it is refused on the
    host, before any GPU work."""
    from ufo_gb300 import capi
    lib = capi.load()
    ops = np.zeros((2, 8), dtype=np.int32)
    ops[0] = [10, 0, 0, 0, 0, 0, 0, 0]       # OP_OBSERVE, index 0: valid
    ops[1] = [10, 0, 0, index, 0, 0, 0, 0]   # OP_OBSERVE, index outside [0, 1)
    table = ctypes.c_void_p(1)  # never dereferenced: the op check comes first
    rc = lib.ufo_track_noalloc(capi.ptr(ops), 2, table, 1, 1, 1, None, None, None, 0, 1, 0,
                               0, 0, 1, None, None, None, None)
    assert rc == -1
    assert b'observation index' in lib.ufo_last_error()
