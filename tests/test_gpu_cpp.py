"""The C++ mirror of the crate's API (include/rebop_gb300.hpp) on the GPU, against the oracle."""

import subprocess

import numpy as np
import pytest

from test_host import _build_cpp_mirror

pytestmark = pytest.mark.gpu


def test_cpp_mirror_runs_bit_exact(O, tmp_path):
    import rebop_gb300  # noqa: F401  (builds and loads the library)

    exe = _build_cpp_mirror(tmp_path)
    r = subprocess.run([str(exe), "gpu"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = {ln.split()[0]: ln.split()[1:] for ln in r.stdout.splitlines() if ln.strip()}
    # Gillespie::new_with_seed(.., 777) then advance_until 0.1, 0.25, 0.7
    net = O.dimer_net()
    sp, t, st = [1, 0, 0, 0], 0.0, O.seed_state(777)
    for tm in (0.1, 0.25, 0.7):
        sp, t, st, _, _, _ = net.advance_until(sp, t, st, tm)
    traj = lines["traj"]
    assert float(traj[0]) == t == 0.7
    assert [int(v) for v in traj[1:]] == list(sp)
    # Ensemble::run over 64 seeds
    seeds = np.array([(s * 0x9E3779B97F4A7C15) % (1 << 64) for s in range(1, 65)], dtype=np.uint64)
    ref, ev, tot, _ = net.run_ensemble([1, 0, 0, 0], seeds, 0.5, 5)
    ens = lines["ensemble"]
    assert int(ens[0]) == tot
    assert [int(v) for v in ens[1:]] == ref[5, 3, :].tolist()
