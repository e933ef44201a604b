"""Seeded synthetic workloads with the shapes and value distributions of the benchmark configs.

No public image suite is involved; every input is generated from a seed:
  * blob images: uniform base U[60, 190] plus 8 Gaussian blobs (sigma U[20, 120] px,
    amplitude U[-80, 80], centre uniform in the image) plus N(0, sigma^2 = 4) noise,
    clamped to [0, 255];
  * noise images: U[0, 255] per pixel;
  * constant images: one value U[0, 255] (the degenerate-quality case);
  * database rows: 256-bit vectors with exactly 128 set bits;
  * planted rows: a query hash with d distinct bits flipped (exact distance d).
"""
import numpy as np

IMG = 512


def blob_image(rng):
    base = rng.uniform(60.0, 190.0)
    img = np.full((IMG, IMG), base, np.float32)
    x = np.arange(IMG, dtype=np.float32)
    for _ in range(8):
        cx, cy = rng.uniform(0, IMG, size=2)
        sigma = rng.uniform(20.0, 120.0)
        amp = rng.uniform(-80.0, 80.0)
        gx = np.exp(-((x - cx) ** 2) / (2 * sigma * sigma)).astype(np.float32)
        gy = np.exp(-((x - cy) ** 2) / (2 * sigma * sigma)).astype(np.float32)
        img += np.float32(amp) * np.outer(gy, gx)
    img += rng.normal(0.0, 2.0, size=(IMG, IMG)).astype(np.float32)
    np.clip(img, 0.0, 255.0, out=img)
    return img


def noise_image(rng):
    return rng.uniform(0.0, 255.0, size=(IMG, IMG)).astype(np.float32)


def constant_image(rng):
    return np.full((IMG, IMG), np.float32(rng.uniform(0.0, 255.0)), np.float32)


def blob_images(n, seed=0):
    rng = np.random.default_rng(seed)
    return np.stack([blob_image(rng) for _ in range(n)]) if n else np.zeros((0, IMG, IMG), np.float32)


def mixed_images(n, seed=0, noise_frac=0.25, const_frac=0.05):
    """Blob images with noise_frac replaced by noise and const_frac by constant images.

    Returns (images [n, 512, 512] f32, kind [n] with 0 blob, 1 noise, 2 constant)."""
    rng = np.random.default_rng(seed)
    kind = np.zeros(n, np.int8)
    order = rng.permutation(n)
    n_noise = int(round(n * noise_frac))
    n_const = int(round(n * const_frac))
    kind[order[:n_noise]] = 1
    kind[order[n_noise:n_noise + n_const]] = 2
    imgs = np.empty((n, IMG, IMG), np.float32)
    for i in range(n):
        imgs[i] = (blob_image, noise_image, constant_image)[kind[i]](rng)
    return imgs, kind


def color_images(n, seed=0, channels=3):
    """n RGB8 (channels 3) or RGBA8 (channels 4) images [n, 512, 512, channels] u8: each
    colour channel an independent blob image; alpha (if any) uniform noise, which the
    luma conversion ignores."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, IMG, IMG, channels), np.uint8)
    for i in range(n):
        for c in range(3):
            out[i, :, :, c] = np.clip(np.rint(blob_image(rng)), 0, 255).astype(np.uint8)
        if channels == 4:
            out[i, :, :, 3] = rng.integers(0, 256, (IMG, IMG), dtype=np.uint8)
    return out


def to_u8(imgs):
    return np.clip(np.rint(imgs), 0, 255).astype(np.uint8)


def rows_128(n, seed=0, chunk=1 << 16):
    """n rows of 32 bytes, each with exactly 128 set bits at uniformly random positions."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, 32), np.uint8)
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        keys = rng.random((m, 256), dtype=np.float32)
        idx = np.argpartition(keys, 128, axis=1)[:, :128]
        bits = np.zeros((m, 256), np.uint8)
        np.put_along_axis(bits, idx, 1, axis=1)
        out[s:s + m] = np.packbits(bits, axis=1, bitorder="little")
    return out


def flip_bits(h, d, rng):
    """Copy of 32-byte hash h with exactly d distinct bits flipped."""
    out = h.copy()
    if d:
        pos = rng.choice(256, size=d, replace=False)
        for p in pos:
            out[p // 8] ^= np.uint8(1 << (p % 8))
    return out


def plant(rows, queries, n_plant, dmin, dmax, seed=0):
    """Overwrite n_plant random rows with copies of random queries at distances U{dmin..dmax}.

    Returns (row positions, query ids, distances) of the planted rows."""
    rng = np.random.default_rng(seed)
    pos = rng.choice(rows.shape[0], size=n_plant, replace=False)
    qid = rng.integers(0, queries.shape[0], size=n_plant)
    dist = rng.integers(dmin, dmax + 1, size=n_plant)
    for p, q, d in zip(pos, qid, dist):
        rows[p] = flip_bits(queries[q], int(d), rng)
    return pos, qid, dist


def plant_near_duplicates(rows, hashes, n_plant, seed, dmax=31):
    """The screening workload's database edit, in place: n_plant rows (at most all of them)
    replaced by copies of randomly chosen hashes ([..., 32] u8, e.g. all 8 dihedral hashes
    of a batch) at exact distances U{0..dmax}. Returns (positions, hash ids, distances)."""
    h = np.ascontiguousarray(hashes, np.uint8).reshape(-1, 32)
    return plant(rows, h, min(int(n_plant), rows.shape[0]), 0, dmax, seed)


def popcount_rows(rows):
    return np.unpackbits(np.ascontiguousarray(rows, np.uint8), axis=1).sum(axis=1)
