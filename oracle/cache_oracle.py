"""FP64 restatement of the learned radiance cache -- test infrastructure.

Only the tests may import this module; it is the checker of the cache's
CUDA kernels, never part of the product path.

The reference (gamalik/cuda-photon-mapper) has no learned component: every
pixel of its photon_mapping_kernel (photonMappingKernel.cu:1409) is shaded
from the photon grid. The cache is this project's own addition, so the
oracle restates the cache's definition rather than reference code:
  * encoding: 16-level multiresolution hash grid (the instant-NGP spatial
    hash x*1 ^ y*2654435761 ^ z*805459861 mod 2^log2_table, dense indexing
    while (res+1)^3 fits a level), trilinear weights, fp16 table values;
    real spherical harmonics of the view direction (degrees 0..3); facing
    normal; a kind flag; a constant 1;
  * network: 4 x [64 x 64, ReLU] then [64 x 16], no biases;
  * loss: relative L2 sum_c (y_c - t_c)^2 / (y_c^2 + eps), y_c held
    constant in the denominator, averaged over 3 x batch.
mlp_step(..., bf16=True) rounds operands to bf16 exactly where the tensor
cores consume them (inputs, weights, hidden activations, dL/dy, activation
gradients) and keeps everything else in float64, so its gradients match the
GPU's up to fp32 accumulation order. bf16=False is the plain FP64 model
whose gradients the finite-difference test checks.
"""
import numpy as np

PRIME_Y = 2654435761
PRIME_Z = 805459861
REL_EPS = 0.01
KNONE = 0x7FFFFFFF

SH_C = (0.28209479177387814, 0.48860251190291987, 1.0925484305920792, 0.94617469575755997,
        0.31539156525251999, 0.54627421529603959, 0.59004358992664352, 2.8906114426405538,
        0.45704579946446572, 0.3731763325901154, 1.4453057213202769)


def bf16(x):
    """Round to the nearest bf16 (ties to even), returned as float64."""
    x32 = np.asarray(x, np.float64).astype(np.float32)
    b = x32.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def grid_box(box_min, box_max):
    """(lo, inv_size) mapping the scene box with a 1 % margin onto [0,1]^3,
    in float32 as the library computes them."""
    bmin = np.asarray(box_min, np.float32)
    ext = np.asarray(box_max, np.float32) - bmin
    m = np.float32(0.01) * np.where(ext > 0, ext, np.float32(1))
    lo = bmin - m
    size = ext + np.float32(2) * m
    return lo, (np.float32(1) / size).astype(np.float32)


def unit_pos(xyz, lo, inv_size):
    """Position in [0,1]^3; float32 inputs are mapped in float32 (the
    kernels' arithmetic), float64 inputs in float64."""
    xyz = np.asarray(xyz)
    if xyz.dtype == np.float32:
        return np.clip((xyz - np.float32(lo)) * np.asarray(inv_size, np.float32), 0, 1).astype(np.float32)
    return np.clip((xyz - lo) * inv_size, 0.0, 1.0)


def level_corners(p, r, log2_t):
    """Slots (n, 8) and trilinear weights (n, 8) of the corners around p
    (the cell position in p's precision, the weights in float64)."""
    p = np.asarray(p)
    f = p * p.dtype.type(r)
    i = np.minimum(np.floor(f).astype(np.int64), r - 1)
    t = (f - i.astype(p.dtype)).astype(np.float64)
    stride = r + 1
    dense = stride ** 3 <= (1 << log2_t)
    idx = np.zeros((len(p), 8), np.int64)
    w = np.zeros((len(p), 8), np.float64)
    for c in range(8):
        o = np.array([c & 1, (c >> 1) & 1, c >> 2])
        cx, cy, cz = (i + o).T.astype(np.uint64)
        if dense:
            idx[:, c] = (cx + stride * (cy + stride * cz)).astype(np.int64)
        else:
            h = (cx ^ ((cy * np.uint64(PRIME_Y)) & np.uint64(0xFFFFFFFF))
                 ^ ((cz * np.uint64(PRIME_Z)) & np.uint64(0xFFFFFFFF)))
            idx[:, c] = (h & np.uint64((1 << log2_t) - 1)).astype(np.int64)
        wt = np.where(o == 1, t, 1.0 - t)
        w[:, c] = wt[:, 0] * wt[:, 1] * wt[:, 2]
    return idx, w


def encode_hash(p, table16, res, log2_t):
    """(n, 2L) hash-grid features; table16 = fp16-rounded table (L, T, 2)."""
    out = np.zeros((len(p), 2 * len(res)))
    for l, r in enumerate(res):
        idx, w = level_corners(p, int(r), log2_t)
        out[:, 2 * l:2 * l + 2] = np.einsum("nc,ncf->nf", w, table16[l][idx])
    return out


def sh16(d):
    x, y, z = np.asarray(d, np.float64).T
    xx, yy, zz = x * x, y * y, z * z
    c = SH_C
    return np.stack([
        np.full_like(x, c[0]), -c[1] * y, c[1] * z, -c[1] * x,
        c[2] * x * y, -c[2] * y * z, c[3] * zz - c[4], -c[2] * x * z, c[5] * (xx - yy),
        c[6] * y * (-3 * xx + yy), c[7] * x * y * z, c[8] * y * (1 - 5 * zz),
        c[9] * z * (5 * zz - 3), c[8] * x * (1 - 5 * zz), c[10] * z * (xx - yy),
        c[6] * x * (-xx + 3 * yy)], axis=1)


def facing_normals(obj, xyz, wo, spheres, plane_axes):
    """Facing normal of diffuse queries (zero rows for volume queries)."""
    n = np.zeros((len(obj), 3))
    for i, o in enumerate(obj):
        if o == KNONE:
            continue
        if o >= 0:
            v = xyz[i] - spheres[o][:3]
            v = v / np.linalg.norm(v)
        else:
            v = np.zeros(3)
            v[plane_axes[-1 - o]] = 1.0
        n[i] = v if np.dot(v, -wo[i]) < 0 else -v
    return n


def features(qa, qd, lo, inv_size, table, res, log2_t, spheres, plane_axes):
    """(n, 64) network inputs of query records (qa, qd as float32 arrays)."""
    qa = np.asarray(qa, np.float32)
    obj = qa[:, 3].view(np.int32)
    xyz = qa[:, :3].astype(np.float64)
    wo = np.asarray(qd, np.float64)[:, :3]
    table16 = np.asarray(table, np.float32).astype(np.float16).astype(np.float64)
    x = np.zeros((len(qa), 64))
    L = len(res)
    x[:, :2 * L] = encode_hash(unit_pos(qa[:, :3], lo, inv_size), table16, res, log2_t)
    x[:, 32:48] = sh16(wo)
    x[:, 48:51] = facing_normals(obj, xyz, wo, spheres, plane_axes)
    x[:, 51] = (obj != KNONE).astype(np.float64)
    x[:, 52] = 1.0
    return x


def split_weights(w):
    w = np.asarray(w, np.float64)
    layers = [w[l * 4096:(l + 1) * 4096].reshape(64, 64) for l in range(4)]
    layers.append(w[4 * 4096:].reshape(64, 16))
    return layers


def mlp_step(x, w, target, bf16_ops=True, den_y=None, eps=REL_EPS):
    """Forward + backward of the loss over the batch.

    x (n, 64) inputs, w flat weights, target (n, 3) already scaled. The
    denominators use den_y (n, 3) when given, else this pass's own outputs
    (held constant either way). Returns dict y (n, 3), loss, w_grad (flat),
    dx (n, 64)."""
    r = bf16 if bf16_ops else (lambda a: np.asarray(a, np.float64))
    W = [r(m) for m in split_weights(w)]
    n = len(x)
    h = [r(x)]
    for l in range(4):
        h.append(r(np.maximum(h[l] @ W[l], 0.0)))
    y = (h[4] @ W[4])[:, :3]
    t = np.asarray(target, np.float64)
    yd = y if den_y is None else np.asarray(den_y, np.float64)
    den = yd * yd + eps
    loss = np.sum((y - t) ** 2 / den) / (3 * n)
    gy = np.zeros((n, 16))
    gy[:, :3] = 2.0 * (y - t) / den / (3 * n)
    gy = r(gy)
    dW = [None] * 5
    dW[4] = h[4].T @ gy
    dz = r((gy @ W[4].T) * (h[4] > 0))
    for l in range(3, 0, -1):
        dW[l] = h[l].T @ dz
        dz = r((dz @ W[l].T) * (h[l] > 0))
    dW[0] = h[0].T @ dz
    dx = dz @ W[0].T
    flat = np.concatenate([m.reshape(-1) for m in dW])
    return {"y": y, "loss": loss, "w_grad": flat, "dx": dx}


def table_grad(p_unit, dx, res, log2_t):
    """Scatter of dL/d(hash features) into a (L, 2^log2_t, 2) table gradient."""
    g = np.zeros((len(res), 1 << log2_t, 2))
    for l, r in enumerate(res):
        idx, w = level_corners(p_unit, int(r), log2_t)
        for c in range(8):
            np.add.at(g[l], idx[:, c], w[:, c:c + 1] * dx[:, 2 * l:2 * l + 2])
    return g


def loss_fixed_den(x, w, target, den_y):
    """FP64 loss with the denominators frozen at den_y (finite differences)."""
    return mlp_step(x, w, target, bf16_ops=False, den_y=den_y)["loss"]
