"""GPU test of the allocation-free Morton sort (hx_lbvh_sort_noalloc).

Callers that cannot allocate device memory (an engine that owns every
device byte through its own allocator, a process that may not grow its
footprint, a latency-critical thread) pass their own device buffers; the
entry point keeps all scratch in a fixed array inside the library.  This
test calls it through the C-ABI on buffers the test owns (allocated by
torch, as a stand-in for the caller's allocator) and checks, on two calls in
a row, that it returns exactly the Morton codes and stable sort order that
hx_scene_upload computes for the same triangles (integer outputs: the
tolerance is bit-exact), from the smallest scene up to exactly 2^18
triangles, where the fixed scratch layout is fullest.  The file sorts last
so a stopping run has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import helios_gb300 as hx
from tests.helpers import TriangleSoupScene, small_icosphere_scene

pytestmark = pytest.mark.gpu


def _world_tris(hs):
    """World-space triangles in flattened order with the device's FP32
    operation order (col0*x + col1*y + col2*z + col3*1, no FMA)."""
    d = hs.desc.contents
    out = []
    for ii in range(d.num_instances):
        inst = d.instances[ii]
        M = np.array(inst.model_matrix[:], np.float32).reshape(4, 4)  # M[col][row]
        mesh = d.meshes[inst.mesh_index]
        verts = np.ctypeslib.as_array(C.cast(mesh.vertices, C.POINTER(C.c_float)), shape=(mesh.num_vertices * 20,))
        pos = verts.reshape(-1, 20)[:, 0:3].astype(np.float32)
        idx = np.ctypeslib.as_array(mesh.indices, shape=(mesh.num_indices,))
        for si in range(mesh.num_submeshes):
            sm = mesh.submeshes[si]
            tri_idx = idx[sm.base_index:sm.base_index + sm.index_count].reshape(-1, 3)
            p = pos[tri_idx]  # (t, 3, 3)
            w = np.empty_like(p)
            for r in range(3):
                acc = M[0][r] * p[..., 0]
                acc = acc + M[1][r] * p[..., 1]
                acc = acc + M[2][r] * p[..., 2]
                acc = acc + M[3][r] * np.float32(1.0)
                w[..., r] = acc
            out.append(w.reshape(-1, 9))
    return np.ascontiguousarray(np.concatenate(out).astype(np.float32))


def _soup(n, seed=31):
    """n random world-space triangles (the fullest case of the fixed scratch)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-50.0, 50.0, (n, 1, 3))
    return TriangleSoupScene((c + rng.normal(0.0, 0.3, (n, 3, 3))).astype(np.float32))


@pytest.mark.parametrize("which", ["box", "ico", "max"])
def test_lbvh_sort_noalloc_matches_scene_upload(which):
    torch = pytest.importorskip("torch")
    ctx = hx.Context(0)
    if which == "box":
        hs = hx.HostScene(hx.SCENE_BOX)
    elif which == "ico":
        hs = small_icosphere_scene(level=4, quads=5000, pool=4, mask=32)
    else:
        hs = _soup(1 << 18)
    scene = hx.Scene(ctx, hs)
    ref = scene.export_bvh()
    world = _world_tris(hs)
    n = world.shape[0]
    assert n == ref["morton"].size
    if which == "max":
        assert n == 1 << 18
    d_world = torch.from_numpy(world).cuda()
    d_morton = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_sorted = torch.zeros(n, dtype=torch.int32, device="cuda")
    for call in range(2):
        d_morton.fill_(-1)
        d_sorted.fill_(-1)
        torch.cuda.synchronize()
        hx.check(hx.lib().hx_lbvh_sort_noalloc(C.c_void_p(d_world.data_ptr()), n, C.c_void_p(d_morton.data_ptr()),
                                               C.c_void_p(d_sorted.data_ptr()), None))
        torch.cuda.synchronize()
        morton = d_morton.cpu().numpy().view(np.uint32)
        order = d_sorted.cpu().numpy().view(np.uint32)
        assert np.array_equal(morton, ref["morton"]), call
        assert np.array_equal(order, ref["sorted"]), call
    # sizes beyond the fixed scratch are rejected, not run
    st = hx.lib().hx_lbvh_sort_noalloc(C.c_void_p(d_world.data_ptr()), (1 << 18) + 1, C.c_void_p(d_morton.data_ptr()),
                                       C.c_void_p(d_sorted.data_ptr()), None)
    assert st == hx.HX_ERR_INVALID_ARG
    assert b"262144" in hx.lib().hx_last_error_string()
    scene.close()
    ctx.close()
