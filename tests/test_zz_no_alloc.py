"""The allocation-free ensemble entry point, rb_ensemble_run_device_noalloc.

It serves callers that cannot let a library allocate device memory: hosts whose
own pool allocator owns all GPU memory, and latency-critical callers that cannot
take cudaMalloc's implicit device synchronisation.  Such a caller passes its own
input and output buffers; everything the engine needs besides them lives in a
fixed 64 KiB array inside the library.  Here the entry point is called through
the C ABI twice in a row, and each result must equal, bit for bit, what the
allocating entry point rb_ensemble_run_device returns for the same inputs
(integer counts: the same zero tolerance as every parity test of this engine).
The second call checks that the array's leftovers from the first call do not
leak into the next result.  The no-allocation call also runs first on a network
that has never been run, and afterwards that network still holds no per-network
device state, and the device's free memory is the same before and after the
second call.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dimer(rb):
    n = rb.Network(4)
    n.add_reaction(rb.Rate.lma(25.0, [1, 0, 0, 0]), [0, 1, 0, 0])
    n.add_reaction(rb.Rate.lma(1000.0, [0, 1, 0, 0]), [0, 0, 1, 0])
    n.add_reaction(rb.Rate.lma(0.001, [0, 0, 2, 0]), [0, 0, -2, 1])
    n.add_reaction(rb.Rate.lma(0.1, [0, 1, 0, 0]), [0, -1, 0, 0])
    n.add_reaction(rb.Rate.lma(1.0, [0, 0, 1, 0]), [0, 0, -1, 0])
    return n


def test_noalloc_entry_point_matches_allocating_one():
    torch = pytest.importorskip("torch")
    import rebop_gb300 as rb
    from rebop_gb300._lib import RB_ERR_INVALID, RB_OK, last_error, lib

    net = _dimer(rb)       # runs through the no-allocation entry point only
    ref_net = _dimer(rb)   # the same network for the allocating entry point
    n, nb, S = 1000, 50, 4
    stream = torch.cuda.current_stream().cuda_stream
    d_x0 = torch.tensor([1, 0, 0, 0], dtype=torch.int64, device="cuda")
    for call in range(2):
        seeds = np.random.default_rng(100 + call).integers(np.iinfo(np.uint64).max, size=n, dtype=np.uint64)
        d_seeds = torch.from_numpy(seeds.view(np.int64)).cuda()
        ref_out = torch.empty((nb + 1, S, n), dtype=torch.int64, device="cuda")
        ref_ev = torch.empty(n, dtype=torch.int64, device="cuda")
        na_out = torch.full((nb + 1, S, n), -7, dtype=torch.int64, device="cuda")
        na_ev = torch.full((n,), -7, dtype=torch.int64, device="cuda")
        status = torch.full((2,), -7, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = lib.rb_ensemble_run_device_noalloc(net._h, n, d_x0.data_ptr(), 0, None, 0, d_seeds.data_ptr(), 1.0,
                                                nb, None, -1, na_out.data_ptr(), na_ev.data_ptr(),
                                                status.data_ptr(), stream)
        assert rc == RB_OK, last_error()
        torch.cuda.synchronize()
        if call == 1:
            # the second call on an already set-up device takes no device memory
            assert torch.cuda.mem_get_info()[0] == free0
        rc = lib.rb_ensemble_run_device(ref_net._h, n, d_x0.data_ptr(), 0, None, 0, d_seeds.data_ptr(), 1.0, nb,
                                        None, -1, ref_out.data_ptr(), ref_ev.data_ptr(), None, stream)
        assert rc == RB_OK, last_error()
        torch.cuda.synchronize()
        assert torch.equal(na_out, ref_out)
        assert torch.equal(na_ev, ref_ev)
        assert int(status[0]) == int(ref_ev.sum()) > n * 1000
        assert int(status[1]) == 0
        # the network that only ran without allocation never built device state
        ev = np.zeros(1, dtype=np.uint64)
        assert lib.rb_ensemble_last_events(net._h, ev.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))) == RB_ERR_INVALID
        assert "no run on this network yet" in last_error()

    # A sampling grid beyond the fixed array is refused with a clear error.
    rc = lib.rb_ensemble_run_device_noalloc(net._h, n, d_x0.data_ptr(), 0, None, 0, d_seeds.data_ptr(), 1.0,
                                            100_000, None, -1, na_out.data_ptr(), None, None, stream)
    assert rc == RB_ERR_INVALID
    assert "no-allocation scratch holds 65536 bytes" in last_error()
