"""bench.py's reference arm: the path on the host cores through the CPU oracle
alone.  It must not load the GPU library, and it must describe the same
workload as the GPU arm (the same signals, block partition and audio)."""
import subprocess
import sys

import numpy as np

ROOT = __file__.rsplit("/tests/", 1)[0]


def test_reference_arm_loads_no_product_library():
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import bench\n"
            "from cochlearmodel_gb300 import native\n"
            "r = bench.RefSweepCPU(n_seeds=1)\n"
            "short = int(np.argmin(r.group_audio))\n"
            "audio = r.step(short, 4)\n"
            "assert audio > 0\n"
            "assert native._LIB is None, 'the product library was loaded'\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert 'libcochlea_gb300' not in maps\n"
            "print('ok', r.units_total, round(r.audio_seconds, 5))\n" % ROOT)
    res = subprocess.run([sys.executable, "-c", "import numpy as np\n" + code],
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    assert res.stdout.startswith("ok")


def test_reference_arm_workload_matches_the_gpu_arm():
    sys.path.insert(0, ROOT)
    import bench
    from cochlearmodel_gb300 import batch, model
    r = bench.RefSweepCPU(n_seeds=4)
    units = audio = 0
    for sp in batch.jnd_sweep_spec(n_seeds=4):
        N, D = batch.block_nodes_for(sp["length"], 1000, 100000)
        prof, _, _ = sp["sweep"].build()
        cfg = model.RunConfig(Time_Block_Length=N / 100000, Decouple_Filter=D,
                              Time_Blocks=len(prof) * D, Overlap_Time=0.005)
        units += len(model.reference_units(cfg))
        audio += len(prof) * N * D / 100000
    assert r.units_total == units == 3025
    assert np.isclose(r.audio_seconds, audio)
    assert len(r.specs) == 24 and sum(len(s["sweep"].powers) + 1 for s in r.specs) == 264


def test_reference_arm_declines_kernel_0_semantics():
    """The host-core arm evaluates kernel 17's semantics only; asked for the
    reference default BM kernel it prints its unavailable line and exits 0."""
    import json
    res = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--bm-kernel", "0"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    line = json.loads(res.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and "unavailable" in line
