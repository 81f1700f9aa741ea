"""Time the reference as shipped on the ensemble workload's grid sizes.

ORACLE directory, measurement script: it imports the unmodified reference
(pvthinker/Fluids2d) with numba, netCDF4, matplotlib and PIL replaced by the
stand-in modules of tests/golden/refstubs.py, so its @njit kernels run as
plain Python floats on one core (numba is installed neither here nor on the
GPU host, and the reference cannot be copied to the GPU host). For each grid
size of the benchmark ensemble (64 .. 512) it builds the first member of that
size of ensemble_case(seed=0) in the reference's own Model, runs the
reference's diag and then `steps` iterations of its run-loop body
(set_dt, step(1)), and times them. The whole-ensemble step time is estimated
as the sum over sizes of (members of that size) x (time of one member step),
the estimator bench.py uses for the port. Writes reference_timing.json next
to this file; bench.py reports it beside its own CPU baseline, labelled with
the host it was measured on.

Usage::

    F2D_REFERENCE_SRC=<reference checkout>/src python oracle/time_reference.py
"""
import json
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

from refstubs import load_reference  # noqa: E402

from fluids2d_gb300 import workloads as wl  # noqa: E402


def _host():
    """CPU model name of this machine (from /proc/cpuinfo where present)."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.machine()


def main(steps=2):
    fd = load_reference()
    members = wl.ensemble_case()
    sizes = sorted({c["nx"] for c in members})
    count = {n: sum(1 for c in members if c["nx"] == n) for n in sizes}
    per_size = {}
    for n in sizes:
        c = next(c for c in members if c["nx"] == n)
        p = fd.Param()
        p.model = "eulerpsi"
        p.nx = p.ny = n
        p.cfl = 0.8
        p.nthreads = 1
        m = fd.Model(p)
        m.mesh.msk[:] = c["msk"]
        m.mesh.finalize()
        m.state.omega[:] = c["fields"]["omega"]
        m.integrator.diag(m.state)
        m.set_dt()
        m.step(1)  # warm-up
        t0 = time.perf_counter()
        for _ in range(steps):
            m.set_dt()
            m.step(1)
        per_size[str(n)] = 1e3 * (time.perf_counter() - t0) / steps
        print(n, f"{per_size[str(n)]:.1f} ms/step", flush=True)
    est_ms = sum(count[n] * per_size[str(n)] for n in sizes)
    cells = sum(c["nx"] * c["ny"] for c in members)
    out = {
        "what": "the reference as shipped (pure-Python kernels: numba absent), one "
                "eulerpsi member of each grid size of ensemble_case(seed=0), "
                f"{steps} timed run-loop iterations each after one warm-up",
        "host": _host(),
        "cores": 1,
        "ms_per_member_step": per_size,
        "members_per_size": {str(n): count[n] for n in sizes},
        "ensemble_ms_per_step": est_ms,
        "value": cells / (est_ms / 1e3),
        "unit": "cell-updates/s",
    }
    with open(os.path.join(HERE, "reference_timing.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
