"""Host logic of bench.py (no GPU): the benchmark case and solver settings it
builds, the .par keys they turn into, the whole-job value of replicas and the
FP64-pipe arithmetic of its roofline entries."""
from __future__ import annotations

import ctypes as C

import pytest

import bench


def test_default_case_is_the_256_cavity_with_the_tuned_mixed_solver():
    vals = bench.bench_case(256, "mg-mixed", None, "quadratic")
    assert (vals["imax"], vals["jmax"], vals["kmax"]) == (256, 256, 256)
    assert vals["re"] == 1000.0 and vals["tau"] == 0.5 and vals["gamma"] == 0.9
    pre, post, inner, omega = bench.MG_SHAPE["mg-mixed"]
    assert (vals["mg_pre"], vals["mg_post"], vals["mg_inner"], vals["mg_omega"]) == \
        (pre, post, inner, omega)
    assert vals["mg_guess"] == "quadratic" and vals["mg_graph"] == 1
    assert vals["solver"] == "mg-mixed"


def test_fp64_arms_are_plain_multigrid_and_the_tuned_shape():
    plain = bench.bench_case(256, "mg", None, "previous")
    assert (plain["mg_pre"], plain["mg_post"], plain["mg_omega"]) == (2, 2, 1.0)
    assert plain["mg_guess"] == "previous"
    tuned = bench.bench_case(256, "mg", None, "quadratic", shape=bench.MG_SHAPE_FP64_TUNED)
    assert (tuned["mg_pre"], tuned["mg_post"], tuned["mg_omega"]) == (1, 2, 1.3)
    # the reference solver: the reference's red-black settings of the 256^3 case
    rb = bench.bench_case(256, "rb", 10000)
    assert rb["solver"] == "rb" and rb["itermax"] == 10000
    assert rb["omg"] == 1.7 and rb["eps"] == 1e-6


def test_bench_keys_parse_in_the_library(nusif_lib, tmp_path):
    """Every extension key the bench writes is accepted by the library's .par
    reader (record mode: an unknown or invalid key would set an error)."""
    from nusif import abi
    from nusif.params import write_par
    vals = bench.bench_case(64, "mg-mixed", None, "quadratic")
    path = write_par(tmp_path / "bench.par", vals)
    p = abi.Parameter()
    nusif_lib.initParameter(C.byref(p))
    nusif_lib.readParameter(C.byref(p), str(path).encode())
    abi.check(nusif_lib)
    assert p.imax == 64 and p.re == 1000.0


def test_replica_value_is_per_job():
    assert bench.replica_value(10.0, 1) == 10.0
    assert bench.replica_value(10.0, 4) == pytest.approx(2.5)


def test_fp64_pipe_fraction():
    # 70 FP64 instructions per cell over 256^3 cells in 2.345 ms
    d = bench._fp64_pipe(70.0, 256 ** 3, 2.345)
    assert d["fp64_inst_per_s"] == pytest.approx(70.0 * 256 ** 3 / 2.345e-3)
    import json
    peaks = bench.ROOT / "MEASURED_PEAKS.json"
    mhz = json.loads(peaks.read_text())["sm_max_mhz"] if peaks.exists() else 2070.0
    assert d["fp64_inst_peak_per_s"] == pytest.approx(bench.FP64_LANES_PER_CLOCK * mhz * 1e6)
    assert 0.0 < d["fp64_pipe_frac"] < 1.0
    assert d["fp64_pipe_frac"] == pytest.approx(d["fp64_inst_per_s"] / d["fp64_inst_peak_per_s"])


def test_headline_network_file():
    """The trained warm-start network the default bench line uses: the flat
    parameter vector of the library's layout and its training record."""
    import numpy as np

    from nusif.learn import saved_meta
    from oracle import unet_oracle as U
    path = bench.NET_PATH
    assert path.exists()
    z = np.load(path, allow_pickle=False)
    assert z["params"].dtype == np.float32 and z["params"].size == U.param_count()
    assert np.all(np.isfinite(z["params"]))
    meta = saved_meta(path)
    assert meta["pairs"] > 0 and "seed" in meta["cases"]


def test_roofline_kernel_is_the_largest_live_share():
    """The line's roofline entry is the kernel with the largest live share of
    the step: launch time x launches per step / ms per step (computeFG once,
    the fine sweep twice per V-cycle, the fine residual once per refinement
    step plus once), not the cold-cache ncu share."""
    roofs = [
        {"kernel": "k_rbgs_sweep_v: sweep", "launch_ms": 0.056, "share_of_step": 0.199},
        {"kernel": "k_mx_residual_df: residual", "launch_ms": 0.146, "share_of_step": 0.088},
        {"kernel": "k_fgh_df: computeFG", "launch_ms": 0.685, "share_of_step": 0.176},
    ]
    bench.live_shares(roofs, "mg-mixed", [4, 4, 4, 5], 2.72, 4)
    by = {r["kernel"].split(":")[0]: r for r in roofs}
    assert by["k_fgh_df"]["launches_per_step"] == 1.0
    assert by["k_rbgs_sweep_v"]["launches_per_step"] == pytest.approx(2 * 4.25)
    # 4 V-cycles: one refinement step (+1); 5: two (+1)
    assert by["k_mx_residual_df"]["launches_per_step"] == pytest.approx((2 + 2 + 2 + 3) / 4)
    assert by["k_fgh_df"]["share_of_step_live"] == pytest.approx(0.685 / 2.72)
    assert bench.dominant(roofs)["kernel"].startswith("k_fgh_df")
    # without live shares the committed list's shares decide
    bare = [dict(r) for r in roofs]
    for r in bare:
        r.pop("share_of_step_live")
    assert bench.dominant(bare)["kernel"].startswith("k_rbgs_sweep_v")
