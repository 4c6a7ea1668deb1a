"""bench.py's JSON line on CPU: the reference arm (the numpy restatement of
the reference's algorithm, timed on the host cores) runs without a GPU, so
its line is checked here against the contract the GPU arm shares: one JSON
line with the metric, the rate, the timing and the CPU-baseline fields, and
ranks other than 0 printing nothing."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env=None, *args):
    env = dict(os.environ)
    env.update(extra_env or {})
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "3",
                        "--steps", "2", "--warmup", "1", *args], capture_output=True, text=True, env=env,
                       timeout=300, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    return [ln for ln in p.stdout.splitlines() if ln.strip()]


def test_reference_arm_line():
    lines = _run()
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "DOF/s" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 1 and d["value"] > 0
    # a timed Arnoldi step extrapolated to the solve, and the line says so
    assert d["extrapolated"] is True and d["its"] > 0 and len(d["t_arnoldi_steps_s"]) == 2
    assert abs(d["t_solve_extrapolated_s"] - d["config"]["dofs"] / d["value"]) <= 1e-9 * d["t_solve_extrapolated_s"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["config"]["dofs"] == 6 * 27 * 20
    assert "small case" in d["config"]["l2_policy"]


def test_reference_arm_other_ranks_print_nothing():
    assert _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []


@pytest.mark.slow
def test_port_extrapolation_against_reference_c2_solve():
    """The reference arm times one preconditioned Arnoldi step of the numpy
    restatement and extrapolates it by the solve's iteration count.  On the
    3D benchmark mesh (48,000 tets) the reference itself was timed here for
    the whole solve (tests/golden/tet20_c2_summary.npz: 120 iterations,
    t_solve, 8 threads).  The port's extrapolated rate on this machine must
    stay within a factor of 3 of that measured rate, and the extrapolation
    formula applied to the reference's own measured stage times (one apply +
    one preconditioner per step) must predict its measured solve within 25%.
    The P1CG values only change numbers, not the work of a step, so the
    set-up here skips the colour probes."""
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    from dg_nn_public_gb300 import element, mesh, sfc
    d = np.load(os.path.join(ROOT, "tests", "golden", "tet20_c2_summary.npz"))
    its, t_solve = int(d["its"]), float(d["t_solve"])
    m = mesh.build_mesh("tet", 20, seed=0)
    order = sfc.hilbert_sfc_order(m.cg_coords)
    from oracle.dg_oracle import OracleDG
    pc = OracleDG(m, element.p3_element(3), element.drst_duv(3)).p1cg()
    cb = bench.CpuBaseline(m, order, element.p3_element(3), rar=np.ones(pc["cola"].size) * 1e-3, smooth=2)
    t_step = min(cb.step() for _ in range(2))
    port = cb.solve_rate(t_step, its)
    ref = m.nele * m.nloc / t_solve
    print("port extrapolated %.1f DOF/s (step %.2f s) vs reference measured %.1f DOF/s: ratio %.2f"
          % (port, t_step, ref, port / ref))
    assert 1.0 / 3.0 <= port / ref <= 3.0
    # the reference's own stage times, extrapolated the same way
    t_ref_step = float(d["t_apply"]) + float(d["t_precond"])
    cycles = -(-its // 30)
    pred = t_ref_step * its + cycles * 2 * float(d["t_apply"])
    print("reference stage times extrapolated: %.1f s vs measured solve %.1f s" % (pred, t_solve))
    assert abs(pred - t_solve) <= 0.25 * t_solve
