"""hg_scan_noalloc, the scan pass for callers that cannot allocate device
memory during a frame (their memory comes from an engine-owned arena or a
fixed budget), against the context-based hg_scan.

The entry point keeps its working memory in a fixed device array, so two calls
in a row must each give hg_scan's result: the second call must not see
anything the first one left behind.  The buffers it is given (inputs and
outputs) are allocated here by the caller, as such a host would.
"""
import ctypes as C

import numpy as np
import pytest

from bevy_hair_gb300 import abi, configs

pytestmark = pytest.mark.gpu


def _lod_and_reference_scan(renderer, sc):
    cam, _ = sc.params()
    renderer.ensure_targets(sc.view.width, sc.view.height, *sc.dom_size)
    g = renderer.upload(sc.mesh)
    renderer.lod(g, cam, abi.SLOT_CAMERA)
    renderer.scan(g, cam, abi.SLOT_CAMERA)
    renderer.synchronize()
    lod_ptr, lod_bytes = g.buffer(abi.SLOT_CAMERA, abi.GBUF_LOD)
    refs = g.read(abi.SLOT_CAMERA, abi.GBUF_REFS)
    indirect = g.read(abi.SLOT_CAMERA, abi.GBUF_INDIRECT)
    return g, lod_ptr, refs, indirect


def test_scan_noalloc_matches_scan_twice_in_a_row():
    import torch

    from bevy_hair_gb300.pipeline import HairRenderer

    lib = abi.load()
    stream = torch.cuda.Stream()
    # two different grooms, so the second call's offsets differ from the first's
    scenes = [configs.config1(scale=0.05), configs.config2(scale=0.02)]
    with HairRenderer(0) as r:
        for sc in scenes:
            g, lod_ptr, want_refs, want_ind = _lod_and_reference_scan(r, sc)
            n_bundles = sc.mesh.bundle_count
            capacity = max(sc.mesh.strand_count(), 1)
            refs = torch.full((capacity * 4,), -1, dtype=torch.int32, device="cuda")  # 0xFFFFFFFF words
            ind = torch.zeros(4, dtype=torch.int32, device="cuda")
            st = lib.hg_scan_noalloc(C.c_void_p(lod_ptr), n_bundles, capacity, C.c_void_p(refs.data_ptr()),
                                     C.c_void_p(ind.data_ptr()), C.c_void_p(stream.cuda_stream))
            assert st == abi.HG_OK
            stream.synchronize()
            got_ind = ind.cpu().numpy().view(np.uint32)
            got_refs = refs.cpu().numpy().view(np.uint32).reshape(-1, 4)
            total = int(want_ind[0])
            assert total > 0
            np.testing.assert_array_equal(got_ind, want_ind)
            np.testing.assert_array_equal(got_refs[:total], want_refs[:total].view(np.uint32).reshape(-1, 4))
            assert (got_refs[total:] == 0xFFFFFFFF).all()  # nothing written past the total
            g.close()


def test_scan_noalloc_rejects_oversized_and_null_inputs():
    lib = abi.load()
    one = C.c_void_p(16)  # never dereferenced: the calls are rejected before any launch
    assert lib.hg_scan_noalloc(one, abi.SCAN_NOALLOC_MAX_BUNDLES + 1, 10, one, one, None) == abi.HG_CAPACITY_EXCEEDED
    assert lib.hg_scan_noalloc(None, 5, 10, one, one, None) == abi.HG_INVALID_ARG
    assert lib.hg_scan_noalloc(one, 5, 10, one, None, None) == abi.HG_INVALID_ARG
    assert lib.hg_scan_noalloc(one, 5, 0, one, one, None) == abi.HG_INVALID_ARG
