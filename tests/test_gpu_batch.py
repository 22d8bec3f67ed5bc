"""GPU tests of the uneven batch driver (files of mixed format, channel count,
length and osamp in one captured CUDA graph), the FFT radix autotuner and
shared stream workspaces.  Parity is against the FP64 streaming oracle, per
file, with the same norm-wise 1e-5 bound as the single-stream tests."""
import numpy as np
import pytest
import torch

from oracle import pfb_oracle as po
from tests.test_gpu_stream import check

pytestmark = pytest.mark.gpu

SMALL = dict(nfiles=6, n1bit=2, nchans=(8, 16, 32), log2_len=(10, 12), osamps=(4, 16),
             acclens=((512, 32), (1024, 64)))


def oracle_vis(f, raw_np):
    ref, _ = po.repfb_xcorr_avg(raw_np, f.channels, acclen=f.acclen, nchunks=f.nchunks, nblock=f.nblock,
                                chanstart=f.chanstart, chanend=f.chanend, osamp=f.osamp, cut=f.cut, bits=f.bits)
    return ref


def as_ref_layout(v):
    """(njobs, M, M, nq) device -> (M, M, nq, njobs) numpy."""
    return v.permute(1, 2, 3, 0).cpu().numpy()


@pytest.fixture(scope="module")
def small_batch():
    from albatros_axion_detection_gb300 import batch
    specs = batch.uneven_batch_specs(seed=11, **SMALL)
    files = batch.files_from_specs(specs, torch.device("cuda", 0))
    return specs, files


def test_uneven_batch_graph_vs_oracle(small_batch):
    from albatros_axion_detection_gb300 import batch
    specs, files = small_batch
    assert {f.bits for f in files} == {1, 4} and len({f.osamp for f in files}) == 2
    bc = batch.BatchCorrelator(files, lanes=3, tune=False).capture()
    try:
        for _ in range(2):  # replays start from reset state each time
            bc.run()
        torch.cuda.synchronize()
        for i, f in enumerate(files):
            check(as_ref_layout(bc.vis(i)), oracle_vis(f, f.raw.cpu().numpy()))
    finally:
        bc.close()


def test_graph_replay_equals_eager_run(small_batch):
    from albatros_axion_detection_gb300 import batch
    _, files = small_batch
    eager = batch.BatchCorrelator(files, lanes=2, tune=False)
    try:
        eager.run()
        torch.cuda.synchronize()
        ref = [eager.vis(i).clone() for i in range(len(files))]
    finally:
        eager.close()
    g = batch.BatchCorrelator(files, lanes=4, tune=False).capture()
    try:
        g.run()
        torch.cuda.synchronize()
        for i in range(len(files)):
            assert torch.equal(g.vis(i), ref[i]), files[i].name
        assert g.launches_per_run() > 0
    finally:
        g.close()


def test_batch_host_copies_in_graph(small_batch):
    """Packets copied from pinned host memory and visibilities copied back,
    both inside the graph."""
    from albatros_axion_detection_gb300 import batch
    specs, _ = small_batch
    files = batch.files_from_specs(specs[:3], torch.device("cuda", 0), host_copies=True)
    ref = []
    for f in files:
        ref.append(oracle_vis(f, f.host.numpy()))
        f.raw.zero_()  # the run must bring the packets in itself
    bc = batch.BatchCorrelator(files, lanes=2, tune=False, vis_to_host=True).capture()
    try:
        bc.run()
        torch.cuda.synchronize()
        assert bc.h2d_bytes == sum(f.raw.numel() for f in files)
        for i in range(len(files)):
            check(bc.vis_host[i].permute(1, 2, 3, 0).numpy(), ref[i])
    finally:
        bc.close()


def test_shared_workspace_matches_private():
    from albatros_axion_detection_gb300 import stream
    from tests.golden import gen
    raw_np = gen.raw_4bit(seed=3, nspec=3 * 512, nchan=8, nant=2)
    raw = torch.from_numpy(raw_np).cuda()
    mk = lambda: stream.StreamCorrelator(2, np.arange(300, 308), 0, 8, 512, 3, 32, 16, 32, nchan_raw=8)
    a, b, c = mk(), mk(), mk()
    try:
        need = b.workspace_bytes()
        assert need > 0
        ws = torch.empty(need, dtype=torch.uint8, device="cuda")
        b.set_workspace(ws)
        c.set_workspace(ws)
        for sc in (a, b, c):  # b and c take turns on the shared scratch
            for j in range(3):
                sc.push(raw, j, final=(j == 2))
        torch.cuda.synchronize()
        assert torch.equal(a.vis_device(), b.vis_device())
        assert torch.equal(a.vis_device(), c.vis_device())
        with pytest.raises(ValueError):
            a.set_workspace(ws[: need // 2])
    finally:
        for sc in (a, b, c):
            sc.close()


def test_workspace_refused_for_unfused_stream():
    from albatros_axion_detection_gb300 import _lib, stream
    sc = stream.StreamCorrelator(1, np.arange(8), 0, 8, 448, 2, 100, 1, 32, nchan_raw=8)  # osamp 1: not fused
    try:
        assert sc.workspace_bytes() == -1
        with pytest.raises(_lib.AlbatrosError):
            sc.set_workspace(torch.empty(1 << 20, dtype=torch.uint8, device="cuda"))
    finally:
        sc.close()


def test_tuned_radix_order_keeps_parity():
    """A forced radix order for the time FFT (n = 576 = 8*8*3*3, reordered)
    gives the oracle's visibilities; clearing it restores the default."""
    from albatros_axion_detection_gb300 import autotune, stream
    from tests.golden import gen
    raw_np = gen.raw_4bit(seed=9, nspec=3 * 1024, nchan=8, nant=1)
    kw = dict(acclen=1024, nchunks=3, nblock=64, chanstart=0, chanend=8, osamp=16, cut=64)
    ref, _ = po.repfb_xcorr_avg(raw_np, np.arange(400, 408), **kw)
    try:
        for order in [(3, 8, 3, 8), (2, 4, 8, 3, 3), (3, 3, 2, 4, 8)]:
            autotune.set_plan(576, order)
            vis, _ = stream.repfb_xcorr_avg(torch.from_numpy(raw_np).cuda(), np.arange(400, 408), **kw)
            check(np.asarray(vis), ref)
    finally:
        autotune.set_plan(576, None)
    with pytest.raises(ValueError):
        autotune.set_plan(576, (8, 8, 8))  # product is not 576


def test_autotuner_picks_and_caches(tmp_path, monkeypatch):
    from albatros_axion_detection_gb300 import autotune
    monkeypatch.setenv("ALBATROS_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    try:
        choice, ms = autotune.tune_time_fft(1024, 64, 16, limit=4)
        assert ms > 0
        assert choice == autotune.BUILTIN or int(np.prod(choice)) == 576
        assert (tmp_path / "tune.json").exists()
        again, ms2 = autotune.tune_time_fft(1024, 64, 16, limit=4)  # cache hit
        assert again == choice and ms2 == ms
    finally:
        autotune.set_plan(576, None)
