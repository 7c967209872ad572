"""The heat kernels decide "latent heat enters cp" as Ts < T < Tl.  The
reference computes the float32 liquid fraction fl = (clip(T, Ts, Tl) - Ts) /
(Tl - Ts) and adds the latent heat where (fl > 0) * (fl < 1)
(jax_am/cfd/gamma.py:12,15).  These checks show the two tests agree for every
float32 T near both edges and across the range, for the workloads' alloy and
for random Ts < Tl <= 2 Ts (no GPU needed)."""
import numpy as np


def _reference_mushy(T, Ts, Tl):
    with np.errstate(invalid="ignore"):
        fl = (np.clip(T, Ts, Tl) - Ts) / (Tl - Ts)
    return (fl > 0) & (fl < 1)


def _kernel_mushy(T, Ts, Tl):
    return (T > Ts) & (T < Tl)


def _near(v, k):
    """The 2k + 1 float32 values closest to v."""
    bits = np.float32(v).view(np.int32)
    return (bits + np.arange(-k, k + 1, dtype=np.int32)).view(np.float32)


def _check(Ts, Tl, rng):
    Ts, Tl = np.float32(Ts), np.float32(Tl)
    T = np.concatenate([_near(Ts, 4096), _near(Tl, 4096),
                        rng.uniform(0.0, 3.0 * float(Tl), 200_000).astype(np.float32),
                        np.array([np.nan, np.inf, -np.inf, 0.0, -1.0], dtype=np.float32)])
    np.testing.assert_array_equal(_kernel_mushy(T, Ts, Tl), _reference_mushy(T, Ts, Tl))


def test_mushy_test_matches_reference_for_the_workload_alloy():
    _check(1563.0, 1623.0, np.random.default_rng(0))


def test_mushy_test_matches_reference_for_random_alloys():
    rng = np.random.default_rng(1)
    for _ in range(200):
        Ts = rng.uniform(200.0, 4000.0)
        Tl = Ts * rng.uniform(1.0 + 1e-6, 2.0)
        _check(Ts, Tl, rng)
