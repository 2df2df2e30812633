"""GPU tests of the per-POI reference prep (k_poi_prepare32).

Where a CTA's 32 queue POIs lie on at most two grid rows and their subsets span few enough
image columns (column and pair walks, subsets up to 64 columns), the CTA forms the mean-independent column sums (grey sum, gradient-product
row moments, S terms) once per image column in shared memory; other CTAs form them per POI.
The same queue in shuffled order puts every CTA on the per-POI path, so equal records for
both orders show that the two paths give the same bits, and that a POI's result does not
depend on where it sits in the queue.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("radius,step,width", [(15, 4, 400), (10, 3, 384), (7, 1, 256), (12, 6, 416), (15, 9, 448),
                                               (20, 4, 400), (30, 5, 448), (31, 9, 448)])
def test_queue_order_does_not_change_results(dic, radius, step, width):
    from fasticgn_gb300 import speckle
    pr = speckle.pair_bumps(seed=500 + radius + step, width=width, height=352, max_disp=6.0, max_strain=0.01)
    q = dic.grid_queue(width, 352, radius, step)
    perm = np.random.default_rng(radius * 100 + step).permutation(len(q))
    outs = []
    for queue in (q.copy(), q[perm].copy()):
        with dic.Engine(radius) as e:
            e.set_ref(pr.ref)
            e.set_tar(pr.tar)
            e.process_pair(queue)
        outs.append(queue)
    in_order, shuffled = outs
    assert (in_order["zncc"] >= 0).mean() > 0.75
    assert in_order[perm].tobytes() == shuffled.tobytes()


def test_rows_straddled_and_partial_ctas(dic):
    """A grid whose rows hold a number of POIs that is not a multiple of 32 (CTAs straddling
    two rows), a queue whose length is not a multiple of 32, and POIs near the image edge
    that fail the entry test, against the same POIs solved one row at a time."""
    from fasticgn_gb300 import speckle
    pr = speckle.pair_bumps(seed=611, width=330, height=300, max_disp=5.0, max_strain=0.01)
    xs, ys = np.meshgrid(np.arange(5, 325, 3, dtype=np.float32), np.arange(10, 295, 7, dtype=np.float32))
    q = dic.make_queue(xs.ravel()[:-5], ys.ravel()[:-5])
    whole = q.copy()
    with dic.Engine(15) as e:
        e.set_ref(pr.ref)
        e.set_tar(pr.tar)
        e.process_pair(whole)
        rows = []
        for y in np.unique(q["y"]):
            part = q[q["y"] == y].copy()
            e.process_pair(part)
            rows.append(part)
    assert np.concatenate(rows).tobytes() == whole.tobytes()
    assert (whole["zncc"] < 0).any() and (whole["zncc"] >= 0).mean() > 0.5
