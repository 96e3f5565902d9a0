"""The CPU restatement of the mesh voxelizer (engine/voxelizer.py) against
analytic inside sets of closed meshes; no GPU needed."""
import numpy as np

from oracle import voxelizer_ref as V
from taichi_elements_gb300 import scenes


def centres(res, dx):
    i, j, k = np.meshgrid(*[np.arange(r) for r in res], indexing="ij")
    return np.stack([(i + 0.5) * dx, (j + 0.5) * dx, (k + 0.5) * dx], -1)


def test_grid_rule():
    assert V.grid_res((24, 40, 64)) == (64, 128, 128)
    assert V.grid_res((32, 32, 32), super_sample=3) == (96, 96, 96)


def test_box_voxels_are_exactly_the_inside_centres():
    res, dx = V.grid_res((32, 32, 32)), 1 / 64
    lo, hi = np.array([0.2, 0.3, 0.25]), np.array([0.6, 0.7, 0.55])
    vox = V.voxelize(scenes.box_mesh(lo, hi), res, dx)
    inside = np.all((centres(res, dx) > lo) & (centres(res, dx) < hi), -1)
    assert vox.min() == 0 and vox.max() == 1
    np.testing.assert_array_equal(vox > 0, inside)


def test_sphere_inside_away_from_the_surface():
    res, dx = V.grid_res((32, 32, 32)), 1 / 64
    vox = V.voxelize(scenes.icosphere((0.5, 0.5, 0.5), 0.3, 4), res, dx)
    d = np.linalg.norm(centres(res, dx) - 0.5, axis=-1)
    far = np.abs(d - 0.3) > 2 * dx
    np.testing.assert_array_equal((vox > 0)[far], (d < 0.3)[far])


def test_padding_columns_stay_empty():
    res, dx = V.grid_res((16, 16, 16)), 1 / 32
    vox = V.voxelize(scenes.box_mesh((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), res, dx, padding=3)
    assert vox[:3].sum() == 0 and vox[-3:].sum() == 0 and vox[:, :3].sum() == 0 and vox[:, :, :3].sum() == 0


def _write_ply(fn, verts, faces, fmt):
    head = [f"ply", f"format {fmt} 1.0", "comment test", f"element vertex {len(verts)}", "property float x",
            "property float y", "property float z", f"element face {len(faces)}",
            "property list uchar int vertex_indices", "end_header"]
    with open(fn, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        if fmt == "ascii":
            for v in verts:
                f.write(f"{v[0]} {v[1]} {v[2]}\n".encode())
            for fc in faces:
                f.write(("3 " + " ".join(map(str, fc)) + "\n").encode())
        else:
            f.write(np.asarray(verts, "<f4").tobytes())
            for fc in faces:
                f.write(np.uint8(3).tobytes() + np.asarray(fc, "<i4").tobytes())


def test_load_mesh_ascii_and_binary(tmp_path):
    from taichi_elements_gb300.mesh_io import load_mesh
    box = scenes.box_mesh((0.1, 0.2, 0.3), (0.4, 0.5, 0.6)).reshape(-1, 3)
    verts, inv = np.unique(box, axis=0, return_inverse=True)
    faces = inv.reshape(-1, 3)
    for fmt in ("ascii", "binary_little_endian"):
        fn = str(tmp_path / f"m_{fmt}.ply")
        _write_ply(fn, verts, faces, fmt)
        tri = load_mesh(fn, scale=2.0, offset=(1.0, 0.0, -1.0))
        want = box.reshape(-1, 9).astype(np.float64) * 2.0 + np.tile([1.0, 0.0, -1.0], 3)
        np.testing.assert_allclose(tri, want, rtol=1e-6, atol=1e-6)
