"""The benchmark's reference arm (the CPU oracle) prints one JSON line with the
keys the benchmark contract names; run on the small c1 workload so it takes
seconds on CPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", "c1",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"] == "c1"
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]


def test_reference_arm_does_not_load_the_gpu_library():
    """The CPU arm builds its inputs with the oracle's generators: the GPU
    library must not be mapped into its process."""
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--config', 'c1', '--steps', '1', "
            "'--warmup', '0']; import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print('GPU_LIB_MAPPED' if 'librschol_gb300' in maps else 'GPU_LIB_ABSENT')")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    assert "GPU_LIB_ABSENT" in out.stdout


def test_roofline_traffic_sources_parse():
    """The bench line's roofline traffic comes from the committed ncu
    summaries: the fused Cholesky's DRAM bytes and algorithmic bytes per c2s
    launch (their ratio scales the traffic to c2), the GEMM launches' bytes."""
    sys.path.insert(0, ROOT)
    import bench
    t, a = bench.traffic_from_profiles("chol_fused_kernel", "c2s")
    assert t and a and 0.1 < t / a < 2.0, (t, a)
    tg, _ = bench.traffic_from_profiles("gemm_tc_kernel", "c2s")
    assert tg and tg > 0
    assert bench.traffic_from_profiles("no_such_kernel", "c2s") == (None, None)
