"""The allocation-free transform (hosnwt_transform_noalloc).

It is for callers that cannot allocate device memory (a host whose GPU
memory is owned by its own pool, or a time loop where cudaMalloc/cudaFree
would synchronise the device).  This file is collected last so that a run
that stops at its first failure has already run every other test.  The
checks call it twice in a row through the C ABI, on device arrays, and
compare with the context-based hosnwt_transform at the transform tolerance.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_noalloc_matches_transform(lib):
    torch = pytest.importorskip("torch")
    import hosnwt
    from oracle.hos_oracle import default_input

    inp = default_input(T_stop=5.0, toler=1e-7, f_out=10.0)
    tank = hosnwt.Tank(inp, 257, 1, 17, 5, 5)  # free-surface grid 257, dealiased grid 771
    info = tank.info()
    rng = np.random.default_rng(5)
    stream = torch.cuda.current_stream().cuda_stream
    calls = [(257, "n", 1, "cos", 3), (771, "big", -1, "sin", 2), (771, "big", 1, "cos", 1),
             (257, "n", -1, "sin", 4)]
    assert info["nd1"] == 771
    for rep in range(2):  # two rounds of calls in a row, sharing the fixed scratch
        for n, grid, direction, cs, nlines in calls:
            host = rng.standard_normal((nlines, n))
            d_in = torch.from_numpy(host).cuda()
            d_out = torch.full_like(d_in, np.nan)
            hosnwt.transform_noalloc(direction, cs, n, nlines, d_in.data_ptr(), d_out.data_ptr(), stream)
            torch.cuda.synchronize()
            got = d_out.cpu().numpy()
            for l in range(nlines):
                ref = tank.transform(grid, direction, cs, "cos", host[l][:, None])[:, 0]
                assert _rel(got[l], ref) < 1e-13 * np.sqrt(n), (rep, n, grid, direction, cs, l)


def test_noalloc_many_lines_and_longest(lib):
    """More lines than one launch takes (the line-group loop runs three
    times, reusing the shared counters and partial sums), and the longest
    length the fixed array admits, against the oracle's transform."""
    torch = pytest.importorskip("torch")
    import hosnwt
    from oracle.hos_oracle import Fourier

    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(9)
    for n, direction, cs, nlines in ((771, 1, "cos", 40), (771, -1, "sin", 40),
                                     (hosnwt.NOALLOC_MAX_N, 1, "cos", 1), (hosnwt.NOALLOC_MAX_N, -1, "sin", 2)):
        F = Fourier(n, 1, n, 1, 4)
        host = rng.standard_normal((nlines, n))
        d_in = torch.from_numpy(host).cuda()
        for rep in range(2):
            d_out = torch.full_like(d_in, np.nan)
            hosnwt.transform_noalloc(direction, cs, n, nlines, d_in.data_ptr(), d_out.data_ptr(), stream)
            torch.cuda.synchronize()
            got = d_out.cpu().numpy()
            for l in range(nlines):
                a = host[l][:, None]
                ref = (F.S2F(a, cs, "cos") if direction == 1 else F.F2S(a, cs, "cos"))[:, 0]
                assert _rel(got[l], ref) < 1e-13 * np.sqrt(n), (rep, n, direction, cs, l)


def test_noalloc_rejects_sizes(lib):
    import hosnwt
    for n in (4, 16386):
        with pytest.raises(hosnwt.HosError):
            hosnwt.transform_noalloc(1, 0, n, 1, 1, 1, 0)
