"""Time the reference's own CUDA kernels (oracle/_ref cubins via refharness) on the
benchmark workloads, for the GPU-baseline comparison.  Test infrastructure only.

    python oracle/time_reference.py --workload iso256            # the whole shot
    python oracle/time_reference.py --workload iso256 --steps 100

Writes the workload's model files to a temporary directory, runs the harness for
the whole shot (or `steps` time steps), with the reference's device
synchronisations, and prints one JSON line: the time loop's CUDA-event time, ms per
time step, Gpts/s over the updated region, and the SM clocks sampled meanwhile.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="iso256", choices=["iso256", "2o128", "vti384", "tti256"])
    ap.add_argument("--steps", type=int, default=0, help="time steps (default: the whole shot)")
    args = ap.parse_args()
    import bench
    cfgd, models, shot, meta = bench.workload(args.workload)
    eng = cfgd["physics"]
    steps = args.steps or cfgd["nt"]
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "case.txt"), "w") as f:
            f.write(f"engine {eng}\nnx {cfgd['nx']}\nny {cfgd['ny']}\nnz {cfgd['nz']}\n")
            f.write(f"dx {cfgd['dx']}\ndy {cfgd['dy']}\ndz {cfgd['dz']}\n")
            f.write(f"sx {shot[0]}\nsy {shot[1]}\nsz {shot[2]}\nnt {cfgd['nt']}\n")
            f.write(f"dt {cfgd['dt']!r}\nfm {cfgd['fm']}\nwtype 1\nmute 0\n")
        for k, a in models.items():
            a.tofile(os.path.join(d, f"{k}.bin"))
        with bench.ClockSampler(0) as clk:
            r = subprocess.run([os.path.join(HERE, "_build", "refharness"), os.path.join(HERE, "_ref"), d,
                                str(steps)], capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stderr)
            raise SystemExit(r.returncode)
        ms = float(r.stdout.split("ms=")[1].split()[0])
    cells = bench.updated_cells(cfgd)
    line = {"workload": meta["workload"], "impl": "reference_cuda_sm103a", "steps": steps, "nt": cfgd["nt"],
            "loop_ms": ms, "ms_per_time_step": ms / steps, "gpts": cells * steps / (ms / 1000.0) / 1e9,
            "clocks": clk.summary()}
    if steps == cfgd["nt"]:
        line["shot_s"] = ms / 1000.0
    print(json.dumps(line))


if __name__ == "__main__":
    main()
