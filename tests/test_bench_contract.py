"""bench.py's host-side pieces, without a GPU: the figures it takes from the committed ncu
summary and the workload description it prints. The numbers in profiles/ and the
bench line must be the same capture's."""
import importlib.util
import os
import re

import numpy as np

from pxdock_gb300 import model, synth

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(REPO, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_profile_figures_match_the_summary_table():
    bench = load_bench()
    text = open(os.path.join(REPO, "profiles", "lbfgs_kernel_ncu.md")).read()
    wipe, tpe = bench.ncu_warp_instructions_per_eval(), bench.ncu_traffic_per_eval()
    assert wipe is not None and tpe is not None
    # the table's instruction count over the evaluations of the captured launch
    inst = float(re.search(r"smsp__inst_executed\.sum \| ([0-9,]+) ", text).group(1).replace(",", ""))
    evals = float(re.search(r"made 8,192 x ([0-9.]+) = ", text).group(1)) * 8192
    assert abs(inst / evals - wipe) <= 1.0
    rd, wr = (float(v.replace(",", "")) for v in
              re.search(r"dram__bytes_write\.sum \| ([0-9,.]+) MB \+ ([0-9,.]+) MB", text).groups())
    assert abs((rd + wr) * 1e6 / evals - tpe) <= 1.0


def test_config_names_the_workload():
    bench = load_bench()
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    box = model.make_box((0.0, 0.0, 0.0), (bench.BOX_SIZE,) * 3, bench.SPACING)
    cfg = bench.config_dict(lig, box)
    assert cfg["workload"].startswith("batched L-BFGS pose optimisation")
    assert cfg["poses"] == bench.N_POSES == 65536
    assert cfg["grid_points"] == int(np.prod(list(box.npoints))) == 81 ** 3
    assert not any(k in cfg for k in ("model", "global_batch", "seq_len"))
    assert bench.config_dict(lig, box, world=2)["parallelism"].startswith("replicas x2")
