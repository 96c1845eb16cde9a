"""Seeded synthetic volumes for the benchmark workloads and the tests.

The reference ships no data (its configs name an ionization dataset that is
not distributed); these generators produce float32 volumes with the shapes and
value distributions of the benchmark configurations.  Arrays are (X, Y, Z)
C-ordered, i.e. the reference's flattened img order (z fastest).
"""
import numpy as np


def gaussian_blobs(shape, count, seed, sigma=(4.0, 12.0), amp=(0.5, 1.5)):
    """Sum of `count` isotropic Gaussians a*exp(-|x-c|^2/(2 s^2)); centres uniform
    in the volume, s uniform in `sigma` (voxels), a uniform in `amp`."""
    rng = np.random.default_rng(seed)
    X, Y, Z = shape
    c = rng.uniform(0, 1, size=(count, 3)) * np.array([X, Y, Z])
    s = rng.uniform(sigma[0], sigma[1], size=count)
    a = rng.uniform(amp[0], amp[1], size=count)
    x = np.arange(X, dtype=np.float64)[:, None, None]
    y = np.arange(Y, dtype=np.float64)[None, :, None]
    z = np.arange(Z, dtype=np.float64)[None, None, :]
    out = np.zeros(shape, dtype=np.float64)
    for k in range(count):
        g = np.exp(-((x - c[k, 0]) ** 2) / (2 * s[k] ** 2))
        g = g * np.exp(-((y - c[k, 1]) ** 2) / (2 * s[k] ** 2))
        g = g * np.exp(-((z - c[k, 2]) ** 2) / (2 * s[k] ** 2))
        out += a[k] * g
    return out.astype(np.float32)


def power_law_field(shape, exponent, seed):
    """Gaussian random field: white noise filtered to power spectrum k^-exponent,
    k=0 removed, normalised to zero mean and unit variance."""
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(shape)
    spec = np.fft.rfftn(noise)
    kx = np.fft.fftfreq(shape[0])[:, None, None]
    ky = np.fft.fftfreq(shape[1])[None, :, None]
    kz = np.fft.rfftfreq(shape[2])[None, None, :]
    k = np.sqrt(kx * kx + ky * ky + kz * kz)
    k[0, 0, 0] = 1.0
    amp = k ** (-exponent / 2.0)
    amp[0, 0, 0] = 0.0
    field = np.fft.irfftn(spec * amp, s=shape, axes=(0, 1, 2))
    field -= field.mean()
    field /= field.std()
    return field.astype(np.float32)


def inside_isovalues(vol, n):
    """n isovalues evenly spaced strictly inside (min, max)."""
    lo, hi = float(np.min(vol)), float(np.max(vol))
    return np.array([lo + (i + 1) * (hi - lo) / (n + 1) for i in range(n)], dtype=np.float32)


def config1(seed=1000):
    """64^3 sum of 8 blobs, 32 isovalues inside the range, 128 bins."""
    vol = gaussian_blobs((64, 64, 64), 8, seed)
    return vol, inside_isovalues(vol, 32), 128


def config2(seed=2000):
    """128^3 k^-3 Gaussian random field, 100 isovalues in [-2.5, 2.5], 256 bins."""
    vol = power_law_field((128, 128, 128), 3.0, seed)
    return vol, np.linspace(-2.5, 2.5, 100).astype(np.float32), 256


def config3(seed=3000, size=256, n=256):
    """size^3: 12 blobs (sigma scaled with the volume) plus 0.05 x unit-variance
    k^-2 noise, n isovalues inside the range, 256 bins."""
    scale = size / 64.0
    vol = gaussian_blobs((size, size, size), 12, seed, sigma=(4.0 * scale, 12.0 * scale))
    vol = vol + 0.05 * power_law_field((size, size, size), 2.0, seed + 1)
    vol = vol.astype(np.float32)
    return vol, inside_isovalues(vol, n), 256
