"""Host logic of bench.py that needs no GPU: the clock record's parsing (NVML samples and
the nvidia-smi CSV fallback), the rejection-relevant throttle reasons, and the algorithmic
FLOP count the roofline divides by."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_clock_summary_from_nvml_samples():
    c = bench.ClockSampler(0)
    # (SM MHz, max MHz, nvmlClocksEventReason bits): power cap in one sample, thermal in one
    c.rows = [(2070.0, 2070.0, 0), (2070.0, 2070.0, 0x4), (1980.0, 2070.0, 0x20), (2070.0, 2070.0, 0)]
    s = c.summary()
    assert s['sm_mhz'] == 2070.0 and s['sm_max_mhz'] == 2070.0 and s['samples'] == 4
    assert s['reasons'] == ['sw_power_cap', 'sw_thermal_slowdown']


def test_clock_summary_from_nvidia_smi_csv():
    c = bench.ClockSampler(0)
    c.rows = []
    c.out = ("0, 2070, 2070, 812.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n"
             "0, 2055, 2070, 1390.1, 0x0000000000000004, Not Active, Not Active, Not Active, Active\n"
             "0, 2070, 2070, 900.0, 0x0000000000000008, Active, Not Active, Not Active, Not Active\n")
    s = c.summary()
    assert s['sm_mhz'] == 2070.0 and s['sm_max_mhz'] == 2070.0 and s['samples'] == 3
    assert s['reasons'] == ['hw_slowdown', 'sw_power_cap']


def test_clock_summary_without_samples():
    c = bench.ClockSampler(0)
    c.rows, c.out = [], ''
    assert c.summary()['reasons'] == ['unsampled']


def test_box_flops_of_the_default_workload(niq):
    # 2 (v + 2) S with v = 3 and S = 3*64 + 3*64*64 + 64 = 12,544 multiply-adds
    params = niq.workloads.spheres_sdf_model()
    assert bench.mlp_macs(params) == 12544
    assert bench.box_flops(params) == 125440


def test_reference_arm_line():
    """`bench.py --impl reference` (the oracle's C/OpenMP tree and marching cubes on the
    host cores) prints one JSON line with the keys the benchmark contract names, for the
    24-bisection tree of the 12-sphere model: 3,677,207 boxes and 264,040 triangles in the
    reference's arithmetic, the counts the GPU's tree gives without outward rounding."""
    import json
    import subprocess
    r = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--steps', '1',
                        '--warmup', '0'], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d['impl'] == 'reference' and d['unit'] == 'boxes/s' and d['higher_is_better'] is True
    assert d['value'] > 0 and d['steps'] == 1
    assert d['details']['boxes_per_step'] == 3677207 and d['details']['triangles_per_step'] == 264040
    assert d['cpu_baseline']['kind'] == 'port' and d['cpu_baseline']['value'] == d['value']
    assert d['e2e'] == {"value": d['value'], "unit": "boxes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
