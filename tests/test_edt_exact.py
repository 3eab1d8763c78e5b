"""The distance transform's exact-comparison passes, run on the host against the oracle.

Maps with both sides <= 4096 take a closed form of the column pass and a row pass whose
breakpoint comparisons are decided with integer cross-multiplication; maps with a side up to
16384 run both passes with those comparisons (rlc_map.cu: edt_col_exact, fh_line_exact).  Both
functions are __host__ __device__: this test compiles them for the host with nvcc, beside the
oracle's C restatement of the reference's Felzenszwalb-Huttenlocher transform, and compares
every cell bit for bit on seeded maps (all densities, 1x1 to 16384 per side, FLT_MAX-heavy
rows), on the reference's benchmark map from the golden fixture and on the generated workload
maps.  The GPU tests check the kernels themselves.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from range_libc_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p if os.path.exists(p) else None


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    d = tmp_path_factory.mktemp("edt_exact")
    orc = d / "rlc_oracle.o"
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-c", os.path.join(ROOT, "oracle", "rlc_oracle.c"),
                           "-o", str(orc)])
    exe = d / "edt_exact_check"
    subprocess.check_call([nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                           "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                           "-I", os.path.join(ROOT, "range_libc_gb300", "csrc"),
                           os.path.join(HERE, "cpp", "edt_exact_check.cu"), str(orc), "-o", str(exe), "-lpthread"])
    return d, exe


def test_exact_passes_equal_the_oracle(harness):
    d, exe = harness
    maps = {"corridor_512": W.corridor_map(512, 5), "rect_disk_1024": W.rect_disk_map(1024, 31),
            "corridor_300x410": np.ascontiguousarray(W.corridor_map(512, 78)[:300, :410])}
    gold = os.path.join(HERE, "golden", "reference_vectors.npz")
    if os.path.exists(gold):
        maps["basement_hallways_5cm"] = np.load(gold)["basement/occ"]
    args = []
    for name, occ in maps.items():
        o = np.ascontiguousarray(occ, np.uint8)
        p = d / f"{name}.u8"
        o.tofile(p)
        args += [str(p), str(o.shape[0]), str(o.shape[1])]
    r = subprocess.run([str(exe), "--quick", *args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith(" 0 mismatches"), r.stdout
