"""The reference arm of the benchmark (`bench.py --impl reference`) times the oracle only: its process
must not load the CUDA library or the host-class library, so that nothing of the product takes part in
the CPU baseline."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_loads_no_product_library(oracle_lib):
    code = (
        "import sys, runpy\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--config', 'small', '--steps', '3', '--warmup', '3']\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('PRODUCT' if ('libtfxgb300' in maps or 'libtressfx_host' in maps) else 'CLEAN')\n"
    )
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = out.stdout.strip().splitlines()
    line = json.loads(lines[-2])
    assert line["impl"] == "reference" and line["cpu_baseline"]["kind"] == "port"
    assert lines[-1] == "CLEAN"
