"""CPU checks of bench.py: the algorithmic byte model behind every GB/s it
reports, and the JSON line of the reference arm (which runs on host cores)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_byte_model_256_32coils():
    sys.path.insert(0, ROOT)
    import bench
    b = bench.algorithmic_bytes(256, 512, 403 * 512, 2, 32)
    img, grid, ks, coords = 32 * 256 ** 2 * 8, 32 * 512 ** 2 * 8, 32 * 206336 * 8, 206336 * 2 * 4
    assert b["interp"] == b["spread"] == grid + ks + coords == 121581568
    assert b["fft"] == 2 * grid and b["pad_deapod"] == b["crop_deapod"] == img + grid
    assert b["step"] == 2 * b["interp"] + 2 * b["fft"] + 2 * (img + grid) == 679370752


def test_pruned_fft_bytes_256_32coils():
    """The four passes of a pruned 512^2 transform pair over 32 coils move
    16.8 + 33.6, 33.6 + 67.1, 67.1 + 33.6 and 33.6 + 16.8 MB."""
    sys.path.insert(0, ROOT)
    import bench
    img, mid, grid = 32 * 256 * 256 * 8, 32 * 256 * 512 * 8, 32 * 512 * 512 * 8
    assert bench.pruned_fft_bytes(256, 512, 32) == (img + mid) + (mid + grid) + (grid + mid) + (mid + img) == 301989888


def test_reference_arm_json_line():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=900, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 1
    assert d["metric"].startswith("NuFFT GB/s") and d["unit"] == "GB/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["e2e"] == {"value": d["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
