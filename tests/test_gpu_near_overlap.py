"""The order-p near field runs on a second stream beside the far field; the
L2P joins the two.  Overlapped and sequential solves give bit-identical
forces and pair sums, for both kernels, in every output mode, through a
captured graph and through the host-buffer entry points."""
import numpy as np
import pytest

from masterthesislucas_gb300 import NBodySolverFMM_SYM_MORTON, datasets

pytestmark = pytest.mark.gpu


def _solve(pos_d, overlap, kernel="gravity", order=8, accumulate=False, scatter=True, **kw):
    import torch
    s = NBodySolverFMM_SYM_MORTON(kernel, max_children=64, theta=0.75, softening=1e-3, order=order, mac="bmax",
                                  near_overlap=overlap, **kw)
    g = torch.full_like(pos_d, 0.25) if accumulate else torch.zeros_like(pos_d)
    t = torch.zeros(1, dtype=torch.float64, device=pos_d.device)
    s.update_tree_device(pos_d)
    s.solve_device(g, t, accumulate=accumulate, scatter=scatter)
    torch.cuda.synchronize()
    st = s.stage_times()
    s.close()
    return g, float(t.item()), st


@pytest.mark.parametrize("kernel,order", [("gravity", 8), ("tsne", 8), ("gravity", 12), ("tsne", 4)])
@pytest.mark.parametrize("accumulate,scatter", [(False, True), (True, False)])
def test_overlap_is_bit_identical(kernel, order, accumulate, scatter):
    import torch
    pos = datasets.two_disks(300000, seed=41).astype(np.float64)
    pd = torch.from_numpy(pos).cuda()
    g0, t0, _ = _solve(pd, False, kernel, order, accumulate, scatter)
    g1, t1, st = _solve(pd, True, kernel, order, accumulate, scatter)
    assert torch.equal(g0, g1) and t0 == t1
    assert torch.isfinite(g1).all() and np.isfinite(t1) and t1 != 0  # gravity: a (negative) potential
    # the split solve reports the near field and the L2P as stages of their own
    assert st["near"] > 0 and st["l2p"] > 0 and st["far"] > 0


def test_overlap_with_tensor_m2l_and_adaptive_orders():
    import torch
    pos = datasets.two_disks(300000, seed=42).astype(np.float64)
    pd = torch.from_numpy(pos).cuda()
    for kw in (dict(centre="box", m2l="tensor"), dict(mac="bmax_adaptive", slack=1.0)):
        mac = kw.pop("mac", "bmax")
        import masterthesislucas_gb300 as m
        res = []
        for ov in (False, True):
            s = m.NBodySolverFMM_SYM_MORTON("gravity", max_children=64, theta=0.7, softening=1e-3, order=8,
                                            mac=mac, near_overlap=ov, **kw)
            g = torch.zeros_like(pd)
            t = torch.zeros(1, dtype=torch.float64, device="cuda")
            s.update_tree_device(pd)
            s.solve_device(g, t)
            torch.cuda.synchronize()
            res.append((g, float(t.item())))
            s.close()
        assert torch.equal(res[0][0], res[1][0]) and res[0][1] == res[1][1]


def test_overlap_in_a_captured_step_matches_the_sequential_solve():
    import torch
    pos = datasets.two_disks(250000, seed=43).astype(np.float64)
    pd = torch.from_numpy(pos).cuda()
    g_ref, t_ref, _ = _solve(pd, False)
    s = NBodySolverFMM_SYM_MORTON("gravity", max_children=64, theta=0.75, softening=1e-3, order=8, mac="bmax")
    g = torch.zeros_like(pd)
    t = torch.zeros(1, dtype=torch.float64, device="cuda")
    s.update_tree_device(pd)
    s.capture_step(pd, g, t, box=np.concatenate([pos.min(0), pos.max(0)]))
    for _ in range(3):
        g.zero_()
        t.zero_()
        s.launch_step()
        torch.cuda.synchronize()
        assert s.async_status() == 0
    # the captured step uses the given box, the reference solve the exact one: same box -> same tree
    g2, t2, _ = _solve(pd, False)
    assert torch.equal(g2, g_ref)
    s.close()
    s2 = NBodySolverFMM_SYM_MORTON("gravity", max_children=64, theta=0.75, softening=1e-3, order=8, mac="bmax",
                                   near_overlap=False)
    gs = torch.zeros_like(pd)
    ts = torch.zeros(1, dtype=torch.float64, device="cuda")
    s2.update_tree_device(pd, pos.min(0), pos.max(0))
    s2.solve_device(gs, ts)
    torch.cuda.synchronize()
    assert torch.equal(g, gs) and float(t.item()) == float(ts.item())
    s2.close()


def test_overlap_through_the_host_buffer_entry_points():
    """tc_update_tree / tc_solve with host buffers: the caller's gradient comes in on the copy stream and
    the near field runs on its own; the sum matches the sequential form bit for bit."""
    from masterthesislucas_gb300.solver import Points
    pos = datasets.two_disks(200000, seed=44).astype(np.float64)
    out = []
    for ov in (False, True):
        s = NBodySolverFMM_SYM_MORTON("gravity", max_children=64, theta=0.75, softening=1e-3, order=8, mac="bmax",
                                      near_overlap=ov)
        pts = Points.from_positions(pos)
        pts.derivative[...] = 0.5
        s.updateTree(pts, pos.min(0), pos.max(0))
        total = s.solveNbody(0.0, pts)
        out.append((pts.derivative.copy(), total, pts.ID.copy()))
        s.close()
    assert np.array_equal(out[0][2], out[1][2])
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]


def test_gradient_buffer_off_a_16_byte_boundary():
    """The L2P writes each particle's force as one 16-byte store when the caller's gradient allows it, two
    8-byte stores otherwise: the same values either way, accumulated or not."""
    import torch
    pos = datasets.two_disks(100000, seed=45).astype(np.float64)
    pd = torch.from_numpy(pos).cuda()
    s = NBodySolverFMM_SYM_MORTON("gravity", max_children=64, theta=0.75, softening=1e-3, order=8, mac="bmax")
    s.update_tree_device(pd)
    n = len(pos)
    for acc in (False, True):
        g_al = torch.full((n, 2), 0.5, dtype=torch.float64, device="cuda")
        flat = torch.full((2 * n + 1,), 0.5, dtype=torch.float64, device="cuda")
        g_off = flat[1:].view(n, 2)
        assert g_al.data_ptr() % 16 == 0 and g_off.data_ptr() % 16 == 8
        t = torch.zeros(1, dtype=torch.float64, device="cuda")
        s.solve_device(g_al, t, accumulate=acc)
        s.solve_device(g_off, t, accumulate=acc)
        torch.cuda.synchronize()
        assert torch.equal(g_al, g_off)
    s.close()


@pytest.mark.parametrize("kernel,order", [("gravity", 8), ("tsne", 4)])
def test_captured_step_with_coarse_far_field_in_the_update(kernel, order):
    """A captured step at depth 10 runs the far field's coarse levels (and the near field's item tables) on a
    side stream of the update, beside its list build; the step's forces and pair sum equal an ordinary
    update + solve bit for bit, replay after replay."""
    import torch
    pos = datasets.two_disks(300000, seed=46).astype(np.float64)
    pd = torch.from_numpy(pos).cuda()
    box = np.concatenate([pos.min(0), pos.max(0)])
    mk = lambda: NBodySolverFMM_SYM_MORTON(kernel, max_children=64, tree_depth=10, theta=0.75, softening=1e-3,  # noqa: E731
                                           order=order, mac="bmax", leaf_p2p=64)
    ref = mk()
    g_ref = torch.zeros_like(pd)
    t_ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    ref.update_tree_device(pd, box[:2], box[2:])
    ref.solve_device(g_ref, t_ref)
    torch.cuda.synchronize()
    assert ref.depth() == 10
    s = mk()
    g = torch.zeros_like(pd)
    t = torch.zeros(1, dtype=torch.float64, device="cuda")
    s.update_tree_device(pd, box[:2], box[2:])
    s.capture_step(pd, g, t, box=box)
    for _ in range(3):
        g.zero_()
        s.launch_step()
        torch.cuda.synchronize()
        assert s.async_status() == 0
        assert torch.equal(g, g_ref) and float(t.item()) == float(t_ref.item())
    # an ordinary solve on the captured handle's tree afterwards still matches (it redoes the coarse levels)
    s.update_tree_device(pd, box[:2], box[2:])
    g2 = torch.zeros_like(pd)
    s.solve_device(g2, t)
    torch.cuda.synchronize()
    assert torch.equal(g2, g_ref)
    ref.close()
    s.close()
