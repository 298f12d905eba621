"""Small hand-built scenes for the traversal tests: scene descriptors of
one triangle mesh, a flat grid whose quads' diagonals give exact ties, and a
cluster of triangles that share one Morton code (one large leaf)."""
import numpy as np


def mesh_desc(pos, idx):
    """A scene descriptor of one triangle mesh (world-space positions, one
    material, no lights); returns it and the arrays it points into."""
    import ctypes as C

    from woodenpbrengine_gb300 import _abi as A

    pos = np.ascontiguousarray(pos, np.float32).ravel()
    idx = np.ascontiguousarray(idx, np.uint32).ravel()
    nt = idx.size // 3
    mesh = A.Mesh(0, nt, 0, 0)
    mat = A.Material()
    mat.type = 0
    mat.alpha_x = mat.alpha_y = 0.2
    d = A.SceneDesc()
    d.n_vertices = pos.size // 3
    d.positions = pos.ctypes.data_as(C.POINTER(C.c_float))
    d.n_triangles = nt
    d.indices = idx.ctypes.data_as(C.POINTER(C.c_uint32))
    d.meshes = C.pointer(mesh)
    d.n_meshes = 1
    d.materials = C.pointer(mat)
    d.n_materials = 1
    for k in range(4):
        d.camera.camera_to_world.m[5 * k] = 1.0
        d.camera.world_to_camera.m[5 * k] = 1.0
    d.camera.fov_deg = 60.0
    d.camera.near_z, d.camera.far_z = 0.1, 1000.0
    d.camera.screen[:] = [-1.0, -1.0, 1.0, 1.0]
    d.camera.res_x = d.camera.res_y = 8
    return C.pointer(d), (pos, idx, mesh, mat)


def grid_desc(n=48):
    """A flat n x n grid of unit quads (2 triangles each) on the plane y = 0
    at integer x, z, and one triangle below it (so the centroid bounds are not
    flat in y). A ray straight down onto a quad's diagonal hits both of its
    triangles at exactly the same t."""
    xs, zs = np.meshgrid(np.arange(n + 1, dtype=np.float32), np.arange(n + 1, dtype=np.float32), indexing="ij")
    grid = np.stack([xs.ravel() - n / 2, np.zeros((n + 1) ** 2, np.float32), zs.ravel() - n / 2], 1)
    below = np.array([[-1.0, -10.0, -1.0], [1.0, -10.0, -1.0], [0.0, -10.0, 1.0]], np.float32)
    v = lambda i, j: i * (n + 1) + j  # noqa: E731
    tris = []
    for i in range(n):
        for j in range(n):
            tris += [v(i, j), v(i + 1, j), v(i + 1, j + 1), v(i, j), v(i + 1, j + 1), v(i, j + 1)]
    m = (n + 1) ** 2
    tris += [m, m + 1, m + 2]
    return mesh_desc(np.concatenate([grid, below]), np.asarray(tris, np.uint32))


def cluster_desc(k, seed=None):
    """k random triangles within 0.004 of (0.5, 0.5, 0.5), far smaller than
    one Morton cell, and one triangle near (1000, 1000, 1000) that stretches
    the centroid bounds: the reference's tree holds the k in one leaf."""
    rng = np.random.default_rng(k if seed is None else seed)
    tris = rng.normal(size=(k, 3, 3)).astype(np.float32)
    tris -= tris.mean(1, keepdims=True)
    tris *= (0.004 / np.abs(tris).max(axis=(1, 2)))[:, None, None]
    tris += np.float32(0.5)
    far = np.array([[[1000, 1000, 1000], [1001, 1000, 1000], [1000, 1001, 1000]]], np.float32)
    return mesh_desc(np.concatenate([tris, far]).reshape(-1, 3), np.arange(3 * (k + 1), dtype=np.uint32))
