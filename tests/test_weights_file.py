"""The committed warm-start parameters (stroemung_gb300/weights/) on the host:
BF16 bit patterns that load as exact FP32 values, one per parameter slot of
the network's flat buffer, all finite, and the benchmark's run_lengths
helper that summarises per-step sweep counts."""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

WEIGHTS = ROOT / "stroemung_gb300" / "weights" / "warmstart_unet_channel_512x128.npy"


def test_bf16_bits_convert_exactly():
    from stroemung_gb300.train_warmstart import bf16_bits_to_f32
    x = np.array([1.0, -2.5, 3.140625, 0.0, -0.0, 1e-30, 6.0e4], dtype=np.float32)
    bits = (x.view(np.uint32) >> 16).astype(np.uint16)   # these values are BF16-exact or truncate
    back = bf16_bits_to_f32(bits)
    assert np.array_equal(back.view(np.uint32), (x.view(np.uint32) >> 16) << 16)


def test_committed_weights_are_finite_bf16_of_the_network_size():
    from stroemung_gb300.train_warmstart import bf16_bits_to_f32
    arr = np.load(WEIGHTS)
    assert arr.dtype == np.uint16
    theta = bf16_bits_to_f32(arr)
    assert np.isfinite(theta).all()
    assert np.abs(theta).max() > 0  # trained, not the zero head alone
    # 4 levels, 3x3 convs, 32/64/128/256 channels: about 1.95 M parameters
    # (plus the layers' padding of K to multiples of 64)
    assert 1.94e6 < arr.size < 2.0e6


def test_run_lengths():
    import bench
    assert bench.run_lengths([]) == []
    assert bench.run_lengths([2000, 2000, 742, 1, 1, 2]) == [[2, 2000], [1, 742], [2, 1], [1, 2]]
