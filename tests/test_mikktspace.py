"""MikkTSpace tangents (world.rs:1238-1260) for meshes without usable
tangents, through ptw_add_mesh: the frame of a flat UV-mapped patch, the
angle-weighted average at welded vertices on a UV sphere against the
analytic tangent, handedness across a mirrored-UV seam, triangles with no
texture area and degenerate triangles."""
import numpy as np

import pathtracer as pt


def mesh_tangents(pos, idx, uv, normals=None, tangents=None):
    w = pt.World.empty()
    mat = w.add_material(pt.default_material())
    w.add_mesh(pos, mat, normals=normals, uvs=uv, tangents=tangents, indices=idx)
    w.build()
    a = w.attributes_raw()[np.argsort(w.bvh_order())].view(np.float32).reshape(-1, 28)
    n = a[:, 1:10].reshape(-1, 3, 3)
    t = a[:, 16:28].reshape(-1, 3, 4)
    w.close()
    return n, t


def test_flat_patch():
    # a 3x3-vertex grid in the xy plane, u along +x, v along +y: tangent +x, orientation-preserving (w negated: -1)
    ys, xs = np.mgrid[0:3, 0:3].astype(np.float32)
    pos = np.stack([xs.ravel(), ys.ravel(), np.zeros(9, np.float32)], 1)
    uv = np.stack([xs.ravel() / 2, ys.ravel() / 2], 1)
    idx = []
    for y in range(2):
        for x in range(2):
            a = y * 3 + x
            idx += [a, a + 1, a + 4, a, a + 4, a + 3]
    nor = np.tile([0, 0, 1], (9, 1)).astype(np.float32)
    _, t = mesh_tangents(pos, np.array(idx), uv, nor)
    np.testing.assert_allclose(t[..., :3].reshape(-1, 3), np.tile([1, 0, 0], (24, 1)), atol=1e-6)
    assert (t[..., 3] == -1).all()
    # u running along -x mirrors the mapping: w flips
    _, t = mesh_tangents(pos, np.array(idx), uv * [-1, 1], nor)
    np.testing.assert_allclose(t[..., :3].reshape(-1, 3), np.tile([-1, 0, 0], (24, 1)), atol=1e-6)
    assert (t[..., 3] == 1).all()


def uv_sphere(nu=48, nv=24):
    pos, nor, uv = [], [], []
    for j in range(nv + 1):
        th = np.pi * j / nv
        for i in range(nu + 1):
            ph = 2 * np.pi * i / nu
            p = [np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)]
            pos.append(p)
            nor.append(p)
            uv.append([i / nu, j / nv])
    idx = []
    for j in range(nv):
        for i in range(nu):
            a, b = j * (nu + 1) + i, (j + 1) * (nu + 1) + i
            idx += [a, b, a + 1, a + 1, b, b + 1]
    return (np.array(pos, np.float32), np.array(nor, np.float32), np.array(uv, np.float32), np.array(idx))


def test_uv_sphere_matches_analytic_tangent():
    pos, nor, uv, idx = uv_sphere()
    n, t = mesh_tangents(pos, idx, uv, nor)
    p = pos[idx].reshape(-1, 3, 3)
    tan = t[..., :3]
    # unit length and in the tangent plane of the vertex normal
    lat = np.abs(p[..., 1]) < 0.95  # away from the poles, where the mapping is singular
    np.testing.assert_allclose(np.linalg.norm(tan[lat], axis=-1), 1, atol=1e-5)
    assert np.abs(np.sum(tan * n, axis=-1))[lat].max() < 1e-5
    # dP/du of the parametrisation: along (-sin phi, 0, cos phi)
    ph = np.arctan2(p[..., 2], p[..., 0])
    want = np.stack([-np.sin(ph), np.zeros_like(ph), np.cos(ph)], -1)
    cosang = np.sum(tan * want, axis=-1)
    # at the u seam (u = 0 and u = 1 are different vertices) only one side's triangles contribute
    seam = np.isin(uv[idx][:, 0].reshape(-1, 3), [0.0, 1.0])
    assert cosang[lat & ~seam].min() > np.cos(np.radians(0.5))
    assert cosang[lat & seam].min() > np.cos(np.radians(4.0))
    # welded vertices (same position, normal, uv) get one frame whichever triangle they belong to
    key = {}
    flat_p, flat_t = p.reshape(-1, 3), t.reshape(-1, 4)
    flat_uv = uv[idx]
    for c in range(len(flat_p)):
        k = tuple(flat_p[c]) + tuple(flat_uv[c])
        if k in key:
            np.testing.assert_array_equal(flat_t[c], flat_t[key[k]])
        else:
            key[k] = c


def test_mirrored_seam_keeps_two_frames():
    # two triangles sharing an edge, the second with mirrored u: different orientation, different handedness
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    uv = np.array([[0, 0], [1, 0], [0, 1], [1, 0], [0, 1], [0, 1]], np.float32)
    uv[3:] = [[1, 0], [2, 1], [0, 1]]
    nor = np.tile([0, 0, 1], (6, 1)).astype(np.float32)
    _, t = mesh_tangents(pos, np.arange(6), uv, nor)
    assert (t[0, :, 3] == -1).all()
    uvm = uv.copy()
    uvm[3:, 0] = 2 - uvm[3:, 0]  # mirror u on the second triangle
    _, t2 = mesh_tangents(pos, np.arange(6), uvm, nor)
    assert (t2[0, :, 3] == -1).all() and (t2[1, :, 3] == 1).all()


def test_zero_area_and_degenerate_triangles():
    # a fan of good triangles around vertex 0 plus one with all uvs equal (no texture area): it takes the
    # group's frame at the shared vertex; a degenerate triangle (two equal positions) copies a good corner
    pos = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [-1, 1, 0], [1, 0, 0]], np.float32)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1], [-1, 1], [1, 0]], np.float32)
    nor = np.tile([0, 0, 1], (6, 1)).astype(np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3, 0, 3, 4, 0, 1, 5])
    uv2 = uv.copy()
    uv2[4] = uv2[3] = [0, 1]  # triangle (0, 3, 4): uvs (0,0), (0,1), (0,1): zero area
    n, t = mesh_tangents(pos, idx, uv2, nor)
    np.testing.assert_allclose(t[..., :3].reshape(-1, 3)[[0, 3]], [[1, 0, 0], [1, 0, 0]], atol=1e-6)
    # the zero-area triangle's corner at vertex 0 (corner 6) has the fan's frame
    np.testing.assert_allclose(t.reshape(-1, 4)[6], t.reshape(-1, 4)[0], atol=1e-6)
    # the degenerate triangle (0, 1, 5) with positions 1 == 5: its corners copy the frames of welded good corners
    np.testing.assert_allclose(t.reshape(-1, 4)[9], t.reshape(-1, 4)[0], atol=0)
    np.testing.assert_allclose(t.reshape(-1, 4)[10], t.reshape(-1, 4)[1], atol=0)


def test_given_tangents_kept_unless_placeholder_or_mixed():
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    uv = np.array([[0, 0], [1, 0], [0, 1]], np.float32)
    nor = np.tile([0, 0, 1], (3, 1)).astype(np.float32)
    given = np.array([[0, 2, 0, 1]] * 3, np.float32)
    _, t = mesh_tangents(pos, np.arange(3), uv, nor, given)
    np.testing.assert_allclose(t[0], [[0, 1, 0, 1]] * 3)  # normalised, handedness as given
    _, t = mesh_tangents(pos, np.arange(3), uv, nor, np.array([[1, 0, 0, 1]] * 3, np.float32))
    np.testing.assert_allclose(t[0], [[1, 0, 0, -1]] * 3, atol=1e-6)  # placeholder: computed instead
    mixed = given.copy()
    mixed[2, 3] = -1
    _, t = mesh_tangents(pos, np.arange(3), uv, nor, mixed)
    np.testing.assert_allclose(t[0], [[1, 0, 0, -1]] * 3, atol=1e-6)
