"""The several-GPU pair path (dic_process_pair_multi, the reference's dual-device queue split,
src/icgn2d1_cuda_mvp.cu:2922-2933) on the one GPU a test box has: two and three engines on
device 0, each solving a row band of the queue from its own host thread, give the same bytes
as one engine.  Each engine's kernels are independent, so sharing one GPU changes only the
timing, never the results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_row_bands_over_engines_equal_one_engine(dic):
    from fasticgn_gb300 import speckle
    pr = speckle.pair_affine(seed=5, width=512, height=384)
    want = dic.grid_queue(512, 384, 15, 5)
    with dic.Engine(15) as e:
        e.set_ref(pr.ref)
        e.set_tar(pr.tar)
        e.process_pair(want)
    for n in (2, 3):
        engines = [dic.Engine(15) for _ in range(n)]
        for e in engines:
            e.set_ref(pr.ref)
            e.set_tar(pr.tar)
        got = dic.grid_queue(512, 384, 15, 5)
        starts = dic.process_pair_multi(engines, got)
        assert starts[0] == 0 and starts[-1] == len(got) and len(starts) == n + 1
        assert got.tobytes() == want.tobytes()
        for e in engines:
            e.close()


def test_multi_reports_an_engine_error(dic):
    a, b = dic.Engine(15), dic.Engine(15)
    rng = np.random.default_rng(1)
    img = rng.integers(0, 255, (128, 128)).astype(np.uint8)
    a.set_ref(img)
    a.set_tar(img)                 # engine b has no images: its band must fail as a state error
    q = dic.grid_queue(128, 128, 15, 8)
    with pytest.raises(RuntimeError):
        dic.process_pair_multi([a, b], q)
    a.close()
    b.close()
