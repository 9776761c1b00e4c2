"""Page-locked host buffers (tg_host_alloc / tg_host_free) for the job API's
copies: a design written from and read into them matches the pageable path bit
for bit.  GPU only."""
import numpy as np
import pytest

from oracle.oracle import cantilever

pytestmark = pytest.mark.gpu


def test_job_copies_through_page_locked_buffers(tg):
    o = cantilever(24, 8, 8)
    pb = tg.Problem(24, 8, 8, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                    list(zip(o.ld_node, o.ld_comp, o.ld_val)))
    job = tg.SimpJob(pb, tg.SimpParams(), tg.SimpOptions(volume_fraction=0.4, filter_radius=1.5,
                                                         max_iterations=4))
    job.step()
    x_ref, xp_ref = job.read()
    xh, xph = tg.host_array(pb.nv), tg.host_array(pb.nv)
    job.read(xh, xph)
    assert np.array_equal(xh, x_ref) and np.array_equal(xph, xp_ref)
    xh[:] = np.clip(0.9 * x_ref + 0.05, 0.0, 1.0)
    job.write_design(xh)
    x2, _ = job.read()
    assert np.array_equal(x2, xh)
    with pytest.raises(ValueError):
        job.read(np.zeros(pb.nv, dtype=np.float32), xph)
    job.close()
    del xh, xph
