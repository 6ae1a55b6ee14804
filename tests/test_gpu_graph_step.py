"""A force step captured as one CUDA graph (tc_step_capture / tc_step_launch)
replays bit-identically to the ordinary update + solve, follows moved
positions inside its box, and flags a point that leaves the box."""
import numpy as np
import pytest

from masterthesislucas_gb300 import NBodySolverFMM_SYM_MORTON, datasets

pytestmark = pytest.mark.gpu


def ordinary(pos_d, order=8, theta=0.8, box=None):
    import torch
    s = NBodySolverFMM_SYM_MORTON("gravity", max_children=64, theta=theta, softening=1e-3, order=order)
    g = torch.zeros_like(pos_d)
    t = torch.zeros(1, dtype=torch.float64, device=pos_d.device)
    if box is None:
        s.update_tree_device(pos_d)
    else:
        s.update_tree_device(pos_d, box[:2], box[2:])
    s.solve_device(g, t)
    torch.cuda.synchronize()
    return s, g.clone(), float(t.item())


def test_replay_matches_ordinary_step():
    import torch
    pos = datasets.two_disks(200000, seed=21).astype(np.float64)
    pd = torch.from_numpy(pos).cuda()
    s, g_ref, t_ref = ordinary(pd)
    g = torch.zeros_like(pd)
    t = torch.zeros(1, dtype=torch.float64, device="cuda")
    box = np.concatenate([pos.min(0), pos.max(0)])
    s.capture_step(pd, g, t, box=box)
    for _ in range(2):
        g.zero_()
        s.launch_step()
        torch.cuda.synchronize()
        assert s.async_status() == 0
        assert torch.equal(g, g_ref)
        assert float(t.item()) == t_ref
    # positions moved inside the captured box: the replay follows them
    moved = pd * 0.999
    pd.copy_(moved)
    s.launch_step()
    torch.cuda.synchronize()
    s2, g2, t2 = ordinary(moved.clone(), box=box)  # the same box, lists built exactly
    assert s.async_status() == 0
    assert torch.equal(g, g2) and float(t.item()) == t2
    # a point outside the box is flagged, never read out of bounds
    pd[0, 0] = 1e3
    s.launch_step()
    torch.cuda.synchronize()
    assert s.async_status() & 1
    s.close()
    s2.close()


def test_capture_needs_a_prior_update():
    import torch
    from masterthesislucas_gb300._lib import TreecodeError
    pos = torch.from_numpy(datasets.two_disks(5000, seed=2).astype(np.float64)).cuda()
    s = NBodySolverFMM_SYM_MORTON("gravity", max_children=64, theta=0.8, order=8)
    g = torch.zeros_like(pos)
    t = torch.zeros(1, dtype=torch.float64, device="cuda")
    with pytest.raises(TreecodeError):
        s.capture_step(pos, g, t)
    s.close()
