"""sg_noise_filter_noalloc -- N^-1 for callers that cannot allocate GPU memory
(their memory belongs to their own pool, they are capturing a CUDA graph, or
they run a real-time loop).  It must give what the regular context-based
sg_noise_filter gives, call after call, while allocating nothing itself: the
test owns every device buffer (torch tensors) and passes raw pointers through
the C ABI, checks that the device's free memory does not move across the
calls, and replays one call captured in a CUDA graph.  This file is collected
last on purpose."""
import numpy as np
import pytest

import sanepic_gb300 as sg
from sanepic_gb300 import build
from sanepic_gb300 import synth

pytestmark = pytest.mark.gpu


def filter_rows(prob, ns):
    """Inverse-noise rows exactly as sg_set_noise derives them (sanepic.cc:533-537)."""
    M = ns // 2
    rows = []
    for ispf in prob["ispf"]:
        k = np.arange(M + 1, dtype=np.float64)
        idx = (k / ispf.size * ns).astype(np.int64)
        spn = ispf[idx] / ns / ns
        spn[0] = ispf[1] * 1e-6 / ns / ns
        rows.append(spn)
    return np.stack(rows)


def rel_rms(got, want):
    return np.sqrt(np.mean((got - want) ** 2)) / np.sqrt(np.mean(want ** 2))


@pytest.mark.parametrize("ns", [4096, 131072])
def test_noalloc_filter_matches_context_filter(ns):
    torch = pytest.importorskip("torch")
    build.build()
    ndet, nseg = 2, 2
    spec = synth.ProblemSpec("noalloc", ndet=ndet, nside=32, nseg=nseg, ns=ns, fknee=0.1,
                             problem=21, precision="f32")
    prob = synth.make_problem(spec, with_tod=False)
    mm = sg.from_problem(prob, precision="f32", with_tod=False)
    x = np.random.default_rng(9).standard_normal(ndet * nseg * ns)
    want = mm.noise_filter(x)
    mm.close()
    filt = torch.tensor(filter_rows(prob, ns), dtype=torch.float32, device="cuda")
    xin = torch.tensor(x, dtype=torch.float32, device="cuda")
    out = torch.empty_like(xin)
    stream = torch.cuda.current_stream().cuda_stream
    # one call per device and tile length before anything is measured or
    # captured: it looks up the static table and prepares the kernel
    assert sg.noise_filter_noalloc(xin.data_ptr(), out.data_ptr(), filt.data_ptr(), ns,
                                   ndet * nseg, nseg, stream) == sg.SG_OK
    for _ in range(2):  # two calls in a row share the static twiddle table
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        rc = sg.noise_filter_noalloc(xin.data_ptr(), out.data_ptr(), filt.data_ptr(), ns,
                                     ndet * nseg, nseg, stream)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert rc == sg.SG_OK
        assert free1 == free0, (free0, free1)  # the call allocated no device memory
        got = out.cpu().double().numpy()  # host copy: no device allocation
        assert rel_rms(got, want) < 2e-6
    # the same call recorded while a CUDA graph is being captured, then replayed
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            rc = sg.noise_filter_noalloc(xin.data_ptr(), out.data_ptr(), filt.data_ptr(), ns,
                                         ndet * nseg, nseg, side.cuda_stream)
    torch.cuda.current_stream().wait_stream(side)
    assert rc == sg.SG_OK
    out.fill_(float("nan"))
    g.replay()
    torch.cuda.synchronize()
    assert rel_rms(out.cpu().double().numpy(), want) < 2e-6
    # a tile longer than the stated maximum is refused, not run
    rc = sg.noise_filter_noalloc(xin.data_ptr(), out.data_ptr(), filt.data_ptr(), 2 * 131072,
                                 1, 1, stream)
    assert rc == sg.SG_ERR_UNSUPPORTED
