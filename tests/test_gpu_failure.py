"""Failure paths on the GPU without a GPU fault: a bounded device wait that
runs out reports SDT_ERR_TIMEOUT and leaves the context usable; the serving
loop cancels queued jobs and its drain gives up after its time limit."""
import ctypes as C

import pytest

import nwchem_gb300 as ng
from nwchem_gb300 import _capi, serve

pytestmark = pytest.mark.gpu

SDT_ERR_STATE, SDT_ERR_TIMEOUT = 4, 6


def test_bounded_wait_runs_out_and_context_survives(cuda_device):
    lib = _capi.lib()
    waited = C.c_double()
    rc = lib.sdt_check_wait_timeout(0.05, C.byref(waited))
    assert rc == SDT_ERR_TIMEOUT
    assert 0.05 <= waited.value < 1.0, waited.value
    assert lib.sdt_check_wait_timeout(2.0, C.byref(waited)) == 1      # longer limits are refused
    # the context still runs work, with the same bits as before
    t = ng.Tiling([3, 4], [5, 6]).with_evl(4)
    files = ng.synth_inputs(t, 4)
    kl = ng.task_list(t)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        a = job.run(kl)
        assert lib.sdt_check_wait_timeout(0.02, C.byref(waited)) == SDT_ERR_TIMEOUT
        b = job.run(kl)
    assert a == b


def test_server_cancel_and_drain_limit(cuda_device):
    specs = serve.job_stream(4, 100.0, 9, 16, 16)
    files = serve.prepare(specs)
    with serve.Server(40 << 30, slots=1) as srv:
        tickets = [srv.submit(s.tiling, f) for s, f in zip(specs, files)]
        srv.cancel(tickets[-1])                     # still queued behind the others
        with pytest.raises(ng.SdtError) as e:
            srv.drain(0.0)                          # the first jobs are still running
        assert e.value.code == SDT_ERR_TIMEOUT
        srv.drain(600)
        st = [srv.status(t) for t in tickets]
        with pytest.raises(ng.SdtError) as e:
            srv.cancel(tickets[0])                  # done: nothing to cancel
        assert e.value.code == SDT_ERR_STATE
    assert [x["state"] for x in st] == [2, 2, 2, -1]
    assert st[-1]["rc"] == SDT_ERR_STATE and "cancelled" in st[-1]["msg"]
