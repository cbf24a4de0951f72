"""bench.py's host-side accounting of the tensor-core stage 1's K-block skip
(no GPU): the fraction of K blocks issued, checked against a direct
restatement over K indices (K index k < kp1 is field row k, real part;
k >= kp1 is field row k - kp1, imaginary part)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _direct(f, width):
    m, n = f.shape
    kp1, kp2 = -(-m // 32) * 32, -(-n // 32) * 32
    g = np.zeros((kp1, kp2), dtype=bool)
    g[:m, :n] = f
    kblocks = 2 * kp1 // 64
    tiles = -(-kp2 // width)
    live = 0
    for t in range(tiles):
        cols = g[:, t * width:(t + 1) * width]
        for kb in range(kblocks):
            rows = [k if k < kp1 else k - kp1 for k in range(64 * kb, 64 * kb + 64)]
            live += bool(cols[rows].any())
    return live / (tiles * kblocks)


@pytest.mark.parametrize('width', [256, 128])
@pytest.mark.parametrize('seed', range(4))
def test_live_fraction_matches_k_index_restatement(width, seed):
    rng = np.random.default_rng(seed)
    m, n = (int(x) for x in rng.integers(40, 700, 2))
    f = np.zeros((m, n), dtype=bool)
    for _ in range(int(rng.integers(1, 4))):          # a few rectangular islands
        r, c = int(rng.integers(0, m)), int(rng.integers(0, n))
        f[r:r + int(rng.integers(1, 60)), c:c + int(rng.integers(1, 60))] = True
    assert bench.stage1_live_fraction(f, width) == pytest.approx(_direct(f, width))


def test_live_fraction_cases():
    assert bench.stage1_live_fraction(np.ones((64, 64)), 256) == 1.0
    two = np.zeros((671, 991), dtype=bool)            # two discs' boxes, 870 columns apart
    two[:121, :121] = True
    two[550:, 870:] = True
    assert bench.stage1_live_fraction(two, 256) == pytest.approx(10 / 84)
    # more than 128 K blocks: the kernel keeps no flags and issues them all
    assert bench.stage1_live_fraction(np.eye(4200, 64, dtype=bool), 256) == 1.0


def test_sample_indices_spread_and_rotate():
    # the reference arm's per-step wavelength samples: n indices spread over
    # the band, shifted by one per step, always inside it
    a = bench.sample_indices(64, 4, 0)
    assert list(a) == [0, 16, 32, 48]
    seen = set()
    for k in range(64):
        idx = bench.sample_indices(64, 4, k)
        assert len(set(idx)) == 4 and idx.min() >= 0 and idx.max() < 64
        seen.update(idx.tolist())
    assert seen == set(range(64))
    assert list(bench.sample_indices(3, 5, 0)) == [0, 1, 2, 3 % 3, 4 % 3]


def test_reference_module_falls_back_to_the_port(monkeypatch, tmp_path):
    # without lentil installed beside the repository the CPU legs run the
    # numpy restatement under oracle/ and say so
    monkeypatch.setattr(bench, 'LENTIL_DIR', str(tmp_path))
    mod, kind, label = bench.reference_module()
    assert kind == 'port' and 'oracle' in label
    for name in ('Pupil', 'Wavefront', 'propagate_dft'):
        assert hasattr(mod, name)


def test_reference_module_uses_lentil_when_installed():
    if not os.path.isfile(os.path.join(bench.LENTIL_DIR, 'lentil', '__init__.py')):
        pytest.skip('lentil is not installed under baseline/_ref')
    mod, kind, label = bench.reference_module()
    assert kind == 'reference' and mod.__version__ in label
