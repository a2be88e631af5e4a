"""Trees of the SSE vox_dot layout (16-byte vox_dot, 128-byte struct
vox_node: a voxvision built with SSE_INTRIN) uploaded through
vox_cuda_tree_upload_layout and searched on the GPU: rays and balls answer
what the reference's SSE build answered on the same trees
(tests/golden/sse_layout.npz) for every ray with a non-zero direction, and
what the scalar build answers for all rays; leaves map back to the caller's
own SSE-layout nodes."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import MISS, load, same_points, sse_tree_from_dump

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

G = load("sse_layout")
CASES = [str(c) for c in G["cases"]]
LAYOUT_SSE = 1


@pytest.fixture(scope="module")
def vg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxvision_gb300.build import build
    build()
    import voxvision_gb300
    return voxvision_gb300


@pytest.mark.parametrize("name", CASES)
def test_sse_layout_tree_searches_on_gpu(vg, name):
    from oracle import oracle as orc
    pre = f"{name}_"
    d = {k[len(pre):]: v for k, v in G.items() if k.startswith(pre)}
    tree = {k[5:]: v for k, v in d.items() if k.startswith("tree_")}
    root, keep = sse_tree_from_dump(tree)
    voxel = np.ascontiguousarray(d["voxel"], np.float32)
    h = C.c_void_p()
    vg.check(vg.lib().vox_cuda_tree_upload_layout(C.c_void_p(root), LAYOUT_SSE, voxel.ctypes.data_as(C.c_void_p),
                                                  C.byref(h)), "vox_cuda_tree_upload_layout")
    dt = vg.DeviceTree(handle=h)
    try:
        leaf, slot, pts = dt.rays(d["ray_origins"], d["ray_dirs"])
        hit = dt.balls(d["ball_centres"], d["ball_radii"])
        ok = ~(d["ray_dirs"] == 0).all(axis=1)       # the builds differ only on all-zero directions
        assert np.array_equal(leaf[ok], d["ray_leaf"][ok])
        assert same_points(pts[ok], d["ray_points"][ok], leaf[ok] != MISS)[0]
        assert np.array_equal(hit, d["ball_hit"])
        orc.set_voxel(tuple(d["voxel"]))
        try:
            ot = orc.OracleTree.from_dump(tree)
            oleaf, _, opts, _ = ot.rays(d["ray_origins"], d["ray_dirs"], nthreads=2)
        finally:
            orc.set_voxel((1, 1, 1))
        assert np.array_equal(leaf, oleaf)
        assert same_points(pts, opts, leaf != MISS)[0]
        # a reported leaf maps back to the caller's own 128-byte node
        k = int(np.nonzero(leaf != MISS)[0][0])
        node = vg.lib().vox_cuda_tree_node(dt.h, int(leaf[k]))
        assert node == root + 128 * int(leaf[k])     # the rebuilt nodes sit in pre-order, 128 bytes apart
    finally:
        dt.close()
    del keep
