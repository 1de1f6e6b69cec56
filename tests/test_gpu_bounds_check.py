"""The parity cases under the bounds-checked build of the library.

The checked build (build_lib.build(bounds_check=True) -> libacqgb300_checked.so) compiles every
instrumented global-memory access of the front end, the tensor-core tile, the column, sign and
rotation stages, the edge-key and extraction kernels with a check against the buffers the
library registered; an access outside all of them is skipped and recorded instead of faulting,
and acq_fetch_results then fails with the site and address. Running the parity suite's small
cases on it (in a child process that loads that library) shows no such access.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# small cases of every path: simple (tensor-core tile + Doppler-group stage, FFT tile, per-step),
# bit-edge search, rotation search (FP32 and tensor-core combine), both noise estimators, IF
CASES = ("test_cfg1_l1ca_4mhz_32prns or test_l1ca_multistep_drift_ci16 or test_l1ca_interm_freq_interp_global_mean "
         "or test_sign_search_two_bits_bit_edge or test_sign_search_odd_doppler_bins_quirk "
         "or test_rotation_l5i_data_bits_multistep or test_rotation_l5i_streamed_ci8 or test_e1b_boc_2_5mhz "
         "or test_l5i_rotation_5mhz_tensor_core_tile or test_tma_and_per_step_column_paths_agree")


def test_parity_cases_under_device_bounds_checks():
    sys.path.insert(0, os.path.join(ROOT, "acquisition.jl_gb300"))
    import build_lib
    build_lib.build(bounds_check=True)
    env = dict(os.environ, ACQ_CHECKED_LIBRARY="1")
    probe = subprocess.run([sys.executable, "-c", "import acqgb300._lib as L; print(L.load().acq_version().decode())"],
                           cwd=os.path.join(ROOT, "acquisition.jl_gb300"), env=env, capture_output=True, text=True)
    assert "bounds-checked" in probe.stdout, probe.stdout + probe.stderr
    r = subprocess.run([sys.executable, "-m", "pytest", "tests/test_gpu_parity.py", "tests/test_gpu_failure.py",
                        "-m", "gpu", "-q", "-p", "no:cacheprovider", "-k", CASES + " or test_column_stage_give_up"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1500)
    print(r.stdout[-3000:])
    assert r.returncode == 0, r.stdout[-6000:] + r.stderr[-3000:]
    assert " passed" in r.stdout and "deselected" in r.stdout
