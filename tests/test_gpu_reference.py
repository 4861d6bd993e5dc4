"""Hogwild quality against the reference's own GPU trainer.

cumf_sgd_ref is singleGPU/ (main.cpp, sgd.cu, sgd_kernel.cu) built unmodified for sm_103a by
oracle/ref_build.sh; its update kernel is sgd_k128_kernel_hogwild_warp32_lrate
(sgd_k128_kernel_hogwild_warp32.h:3-104).  Both trainers get the same 12-byte training file
and the reference's canonical flags (data/netflix/run.sh:3: -l 0.05 -a 0.08 -b 0.3 -k 128
-t 20 -u 1 -v 1 -x 1 -y 1) with -s 52 x SMs (README.md:61, 7,904 workers on 152 SMs); both
models are scored by the same evaluator (calc_rmse, pinned to test/mf.cpp:3815-3839), and
every score is checked against the reference's own mf-predict -e 0 (4 printed decimals).

Bound: 0.002 test RMSE.
  - 480,189 x 17,770, 99M ratings (the benchmark shape): |ours - reference| <= 0.002.
  - 10,000 x 2,000, 0.9M ratings, Zipf(1.0) ids (mean of three runs each): ours <= reference
    + 0.002.  The bound is one-sided here because the two differ by far more than 0.002 in
    our favour at this concurrency: measured 0.84 against 0.92 at 7,904 workers, with about
    12% of all ratings on the most-rated item.  Part of that is the reference's one
    persistent launch for all 20 epochs (this library's kernel run that way measures 0.866
    instead of 0.839), the rest is lost updates of the reference kernel itself.
The reference seeds from time() and clock(), so its runs are not repeatable; the margins
measured on GB300 are several times the run-to-run spread.
"""
import os

import numpy as np
import pytest

import cumf_sgd_gb300 as cm
from cumf_sgd_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "cumf_sgd_gb300", "bin", "cumf_sgd")


@pytest.fixture(scope="module")
def ref_tools():
    from oracle import oracle, ref_tools
    try:
        oracle.build_reference()
    except Exception as e:  # the reference sources are not shipped with a plain checkout
        pytest.skip(f"reference trainer not built: {e}")
    if not ref_tools.available("cumf_sgd_ref"):
        pytest.skip("reference trainer cumf_sgd_ref not built (no reference sources on this host)")
    return ref_tools


def _ours(train_path, model_path, workers, seed, extra=()):
    import subprocess
    from oracle import ref_tools
    cmd = [CLI] + ref_tools.cumf_flags(workers, 20) + ["--seed", str(seed), "--quiet", *extra, train_path, model_path]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-500:] + r.stderr[-500:]


def _compare(ref_tools, spec, tmp_path, reps, extra=()):
    sm, _, _ = cm.device_info(0)
    workers = 52 * sm
    train, test = synth.generate(spec, seed=0, device="cuda")
    tr_path, te_path = str(tmp_path / "train.bin"), str(tmp_path / "test.bin")
    ref_tools.write_records(train, tr_path)
    ref_tools.write_records(test, te_path)
    te = cm.MFProblem.from_arrays(test["u"], test["v"], test["r"])

    def score(model_path):
        got = cm.calc_rmse(te, cm.load_model(model_path))
        if ref_tools.available("mf-predict"):  # the reference's evaluator prints 4 decimals
            assert abs(ref_tools.libmf_rmse(te_path, model_path) - got) <= 6e-5, model_path
        return got

    ref, ours = [], []
    for rep in range(reps):
        mp = str(tmp_path / "ref.model")
        out = ref_tools.run_reference_gpu(tr_path, mp, workers, 20)
        assert out["rc"] == 0 and out["update_per_sec"], out
        ref.append(score(mp))
        mo = str(tmp_path / "ours.model")
        _ours(tr_path, mo, workers, rep + 1, extra)
        ours.append(score(mo))
    return float(np.mean(ref)), float(np.mean(ours)), ref, ours


@pytest.mark.parametrize("extra", [(), ("--hot-rows", "0.5")], ids=["plain", "row-copies"])
def test_hogwild_c2_shape_within_0002_of_reference_kernel(ref_tools, lib, cuda, tmp_path, extra):
    """The default update and the copies of the most-rated rows (--hot-rows 0.5)."""
    ref, ours, r_all, o_all = _compare(ref_tools, synth.C2, tmp_path, reps=1, extra=extra)
    assert abs(ours - ref) <= 0.002, (ours, ref)


def test_hogwild_c1_shape_not_worse_than_reference_kernel(ref_tools, lib, cuda, tmp_path):
    ref, ours, r_all, o_all = _compare(ref_tools, synth.C1, tmp_path, reps=3)
    assert ours <= ref + 0.002, (o_all, r_all)
