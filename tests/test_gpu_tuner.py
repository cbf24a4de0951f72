"""Both pair-tile widths of the tensor-core MFT (256 and 128 output columns)
against the oracle, and the tile-shape autotuner that chooses between them.

Per output element the two widths run the same K-ordered arithmetic (the
width only changes which elements share a tile), so complex results agree
to rounding; intensities reduced over wavelengths with FP32 atomic adds agree
to FP32 rounding of the sum."""
import numpy as np
import pytest
import torch

import lentil_gb300 as lg
from lentil_gb300 import tuner
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu

SPLIT_TOL = {'split-bf16': 3e-5, 'split-fp16': 2e-6}        # random complex fields

# (m, n, M, N): square, rectangular with narrow last tiles of either width,
# a field wider than one 256-column tile, a window of several stage-2 tiles
SHAPES = [(64, 64, 64, 64), (70, 53, 64, 81), (300, 200, 96, 150), (257, 390, 200, 130)]


@pytest.fixture(autouse=True)
def _restore_tuner():
    yield
    tuner.force_tile(0)
    tuner.set_mode('measure')


@pytest.mark.parametrize('precision', ['split-bf16', 'split-fp16'])
@pytest.mark.parametrize('shape', SHAPES)
def test_both_tiles_match_oracle(cuda_device, precision, shape):
    m, n, M, N = shape
    rng = np.random.default_rng(m * 1000 + n)
    f = rng.standard_normal((2, m, n)) + 1j * rng.standard_normal((2, m, n))
    kw = dict(shape=(M, N), shift=(0.3, -1.2), offset=(2, -1), unitary=True)
    alpha = (0.9 / m, 1.1 / n)
    out = {}
    for tile in (256, 128):
        with tuner.forced(tile):
            out[tile] = lg.fourier.dft2_batch(f, alpha, precision=precision, **kw)
            assert tuner.last_tile() == tile
    for k in range(2):
        ref = lo.dft2(f[k], alpha, **kw)
        for tile in (256, 128):
            assert lo.peak_normalised_error(out[tile][k], ref) < SPLIT_TOL[precision], (tile, k)
        assert lo.peak_normalised_error(out[128][k], out[256][k]) < 1e-12


def _small_plan(precision, L=6, batch=2):
    H = 96
    amp = lg.normalize_power(lg.circle((H, H), 44))
    rng = np.random.default_rng(5)
    lam = np.linspace(550e-9, 750e-9, L)
    opd = np.stack([rng.normal(0, 40e-9, (H, H)) * (amp > 0) for _ in range(batch)])
    alphas = [((1 / H) * 6e-6 / (l * 4 * 2),) * 2 for l in lam]
    shifts = [(0.0, 0.0)] * L
    plan = lg.PSFPlan((H, H), (0, 0, H, H), (0, 0), lam, alphas, shifts, (80, 72), (80, 72),
                      (0, 0), batch=batch, precision=precision)
    A = torch.as_tensor(np.stack([amp] * batch), device='cuda')
    O = torch.as_tensor(opd, device='cuda')
    W = torch.full((batch, L), 1.0 / L, dtype=torch.float64, device='cuda')
    return plan, A, O, W


def test_both_tiles_broadband_plan(cuda_device):
    # the intensity epilogue (|F|^2 reduced into the window) at either width
    # equals the complex128 plan
    ref_plan, A, O, W = _small_plan('fp64')
    ref = ref_plan.execute(A, O, W).cpu().numpy()
    plan, A, O, W = _small_plan('split-fp16')
    for tile in (256, 128):
        with tuner.forced(tile):
            img = plan.execute(A, O, W).cpu().numpy()
            assert tuner.last_tile() == tile
        for b in range(2):
            assert lo.peak_normalised_error(img[b], ref[b]) < 2e-6, (tile, b)


@pytest.mark.parametrize('mode', ['measure', 'model'])
def test_tuner_decides_once_per_launch_class(cuda_device, mode):
    tuner.clear()
    tuner.set_mode(mode)
    rng = np.random.default_rng(3)
    f = rng.standard_normal((3, 120, 88)) + 1j * rng.standard_normal((3, 120, 88))
    kw = dict(shape=(100, 70), unitary=False, precision='split-fp16')
    run = lambda x: lg.fourier.dft2_batch(x, (0.008, 0.012), **kw)
    first = run(f)
    if mode == 'measure':
        # the model prices the widths within 1.4x here (one wave either way),
        # so the class is tuned online: four trial launches alternating the
        # widths, the model's first (each returns its result to the host, so
        # all have finished afterwards), then a launch that decides
        widths = [tuner.last_tile()]
        assert tuner.entries() == 0
        for _ in range(3):
            out = run(f)
            widths.append(tuner.last_tile())
            assert tuner.entries() == 0
            assert lo.peak_normalised_error(out, first) < 1e-12   # either width
        assert widths[0] == widths[2] and widths[1] == widths[3] and widths[0] != widths[1]
        run(f)
    assert tuner.entries() == 1
    tile = tuner.lookup(120, 88, 100, 70, 3, 'split-fp16', 'complex')
    assert tile in (128, 256) and tuner.last_tile() == tile
    again = run(f)
    assert tuner.entries() == 1 and tuner.last_tile() == tile
    assert lo.peak_normalised_error(again, first) < 1e-12
    with tuner.forced(tile):                         # the tuned launch is the plain launch
        assert np.array_equal(run(f), again)
    # two fields instead of three occupy the GPU alike: the same class
    run(f[:2])
    assert tuner.entries() == 1 and tuner.last_tile() == tile
    assert tuner.lookup(120, 88, 100, 70, 2, 'split-fp16', 'complex') == tile
    tuner.clear()
    assert tuner.entries() == 0 and tuner.lookup(120, 88, 100, 70, 3, 'split-fp16', 'complex') == 0


def test_model_prefers_wide_tiles_when_the_gpu_is_full(cuda_device):
    # 64 wavelengths of a 256^2 field into a 256^2 window: thousands of tiles
    # at either width, so the model keeps the 256-wide tile; one small
    # transform fills one tile at either width, so it takes the 128-wide one
    tuner.clear()
    tuner.set_mode('model')
    rng = np.random.default_rng(4)
    big = rng.standard_normal((64, 256, 256)) + 0j
    lg.fourier.dft2_batch(big, (1 / 256, 1 / 256), shape=(256, 256), precision='split-bf16')
    assert tuner.lookup(256, 256, 256, 256, 64, 'split-bf16', 'complex') == 256
    small = rng.standard_normal((1, 48, 48)) + 0j
    lg.fourier.dft2_batch(small, (1 / 48, 1 / 48), shape=(48, 48), precision='split-bf16')
    assert tuner.lookup(48, 48, 48, 48, 1, 'split-bf16', 'complex') == 128


def test_capture_uses_model_and_caches_nothing(cuda_device):
    # a plan execute first seen under CUDA-graph capture cannot be timed: it
    # runs with the model's width, caches nothing, and replays correctly
    plan, A, O, W = _small_plan('split-bf16', L=5, batch=1)
    ws = torch.empty(max(1, plan.workspace_bytes(1)), dtype=torch.uint8, device='cuda')
    sub = torch.tensor([0, 2, 4], dtype=torch.int32, device='cuda')
    for tile in (256, 128):              # every kernel used once, outside capture,
        with tuner.forced(tile):         # on another launch shape (3 wavelengths)
            plan.execute(A, O, W[:, :3].contiguous(), lam_idx=sub, workspace=ws)
    tuner.clear()
    tuner.set_mode('measure')
    out = torch.zeros((1, 80, 72), dtype=torch.float64, device='cuda')
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            plan.execute(A, O, W, out=out, check=False, workspace=ws)
    assert tuner.entries() == 0
    g.replay()
    torch.cuda.synchronize()
    for _ in range(5):                              # uncaptured: four trials, then decided
        ref = plan.execute(A, O, W)
        torch.cuda.synchronize()
    assert tuner.entries() == 1
    assert lo.peak_normalised_error(out.cpu().numpy(), ref.cpu().numpy()) < 1e-6


def test_plan_tile_setting(cuda_device):
    # a plan's own width overrides the tuner; 0 hands the choice back
    plan, A, O, W = _small_plan('split-bf16', L=4, batch=1)
    for tile in (128, 256):
        plan.set_tile(tile)
        plan.execute(A, O, W)
        assert tuner.last_tile() == tile
    with tuner.forced(128):                 # a forced width overrides the plan's own
        plan.execute(A, O, W)
        assert tuner.last_tile() == 128
    plan.set_tile(0)
    with tuner.forced(128):
        plan.execute(A, O, W)
        assert tuner.last_tile() == 128
    with pytest.raises(ValueError):
        plan.set_tile(64)


def test_tuner_argument_errors(cuda_device):
    with pytest.raises(ValueError):
        tuner.force_tile(64)
    with pytest.raises(ValueError):
        tuner.set_mode('fastest')


def test_tuner_cache_file_round_trip(cuda_device, tmp_path):
    # decided classes survive a save / clear / load cycle; a file from another
    # kind of GPU (or an unreadable one) is ignored
    import json
    tuner.clear()
    tuner.set_mode('model')
    rng = np.random.default_rng(13)
    f = rng.standard_normal((2, 40, 30)) + 0j
    lg.fourier.dft2_batch(f, 0.02, shape=(32, 36), precision='split-bf16')
    w = tuner.lookup(40, 30, 32, 36, 2, 'split-bf16', 'complex')
    assert w in (128, 256)
    path = tmp_path / 'tiles.json'
    assert tuner.save(str(path)) == tuner.entries() >= 1
    tuner.clear()
    assert tuner.lookup(40, 30, 32, 36, 2, 'split-bf16', 'complex') == 0
    assert tuner.load(str(path)) >= 1
    assert tuner.lookup(40, 30, 32, 36, 2, 'split-bf16', 'complex') == w
    doc = json.loads(path.read_text())
    doc['device']['sm_count'] += 1
    other = tmp_path / 'other.json'
    other.write_text(json.dumps(doc))
    tuner.clear()
    assert tuner.load(str(other)) == 0 and tuner.entries() == 0
    (tmp_path / 'bad.json').write_text('{not json')
    assert tuner.load(str(tmp_path / 'bad.json')) == 0
    assert tuner.load(str(tmp_path / 'missing.json')) == 0


def test_captured_execute_replays_new_inputs(cuda_device):
    # PSFPlan.capture: one CUDA graph of the execute; a replay after writing
    # new inputs into the captured tensors equals a plain execute of them
    plan, A, O, W = _small_plan('split-bf16', L=4, batch=2)
    out = torch.empty((2, 80, 72), dtype=torch.float64, device='cuda')
    cap = plan.capture(A, O, W, out)
    first = cap.replay().clone()
    torch.cuda.synchronize()
    ref = plan.execute(A, O, W)
    assert lo.peak_normalised_error(first.cpu().numpy(), ref.cpu().numpy()) < 1e-6
    O.mul_(1.7)                                     # new inputs, in place
    W[:, 0] = 0.0
    got = cap.replay().clone()
    cap.status()
    ref2 = plan.execute(A, O, W)
    for b in range(2):
        assert lo.peak_normalised_error(got[b].cpu().numpy(), ref2[b].cpu().numpy()) < 1e-6
    assert lo.peak_normalised_error(got[0].cpu().numpy(), first[0].cpu().numpy()) > 1e-3
