"""What the trained proposal network gains over the method without it: after
a short training on particles of a few maps (the library's own kernels),
the rotations it proposes for new particles of those maps lie closer to the
true poses than those of the untrained network."""
import numpy as np
import pytest
import torch

import tg3
from tg3 import learned, synth

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def _nearest(net, ps, n_rot):
    n = len(ps.cls)
    out = torch.empty((n, tg3.Cnn.N_OUT), dtype=torch.float32, device=DEV)
    net.forward(ps.images, out)
    q = torch.empty((n, n_rot, 4), dtype=torch.float64, device=DEV)
    t = torch.empty((n, 1, 2), dtype=torch.float64, device=DEV)
    tg3.Cnn.propose(out, n_rot, 1, 3, q, t)
    torch.cuda.synchronize()
    return learned.angle_deg(q.cpu().numpy(), ps.quat_true[:, None, :]).min(1)


def test_training_brings_proposals_closer_to_the_truth():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    rng = np.random.default_rng(77)
    box, px = 128, 1.4
    maps = [synth.blob_map(rng, 120, (1.5, 3.0), px, 40.0) for _ in range(2)]
    rL = synth.config_rL(box, px)
    train = synth.particle_set(61, maps, np.arange(24000) % 2, box, px, 32, rL, 3.0, 1.0, device=DEV)
    test = synth.particle_set(62, maps, np.arange(400) % 2, box, px, 32, rL, 3.0, 1.0, device=DEV)
    net = tg3.Cnn(0, seed=3)
    try:
        before = _nearest(net, test, 64)
        R = torch.as_tensor(synth.quat_to_mat(train.quat_true).reshape(-1, 9)).to(DEV)
        t = torch.as_tensor(train.trans_true).to(DEV)
        losses = learned.train(net, train.images, R, t, 4, 256, 2e-3, seed=1)
        after = _nearest(net, test, 64)
    finally:
        net.close()
    assert losses[-1] < losses[0]
    # the trained proposals: nearer the truth for the median particle, and
    # within 15 degrees for clearly more particles than before
    assert np.median(after) < 0.8 * np.median(before), (np.median(before), np.median(after))
    assert np.mean(after < 15) > np.mean(before < 15) + 0.05, (np.mean(before < 15), np.mean(after < 15))


def test_matching_training_carries_over_to_unseen_maps():
    """Matching mode: after a short contrastive training on particles of two
    maps, the 64 best-matching of a third, never-seen map's 6,912 references
    hold a rotation within 10 degrees of the truth for most of that map's
    particles; with the untrained network they rarely do."""
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    rng = np.random.default_rng(79)
    box, px, pf = 128, 1.4, 2
    maps = [synth.blob_map(rng, 120, (1.5, 3.0), px, 40.0) for _ in range(3)]
    rL = synth.config_rL(box, px)
    train = synth.particle_set(63, maps[:2], np.arange(24000) % 2, box, px, 32, rL, 3.0, 1.0,
                               device=DEV, with_data=False)
    test = synth.particle_set(64, maps[2:], np.zeros(300, np.int64), box, px, 32, rL, 3.0, 1.0,
                              device=DEV, with_data=False)
    ctx = tg3.Context(0)
    net = tg3.Cnn(0, seed=4)
    try:
        for c, bm in enumerate(maps):
            ctx.set_volume(c, synth.padded_volume(bm, box, pf, device=DEV, dtype=torch.float32), pf)
        refs_train = torch.empty_like(train.images)
        for c in range(2):
            sel = np.nonzero(train.cls == c)[0]
            refs_train[torch.as_tensor(sel, device=DEV)] = learned.render_references(
                ctx, c, train.quat_true[sel], box)
        qg = synth.global_rotations(4, 36)
        grid_refs = learned.render_references(ctx, 2, qg, box)
        qg_d = torch.as_tensor(qg).to(DEV)

        def within10():
            z = learned.reference_embeddings(net, grid_refs)
            out = torch.empty((len(test.cls), tg3.Cnn.N_OUT), dtype=torch.float32, device=DEV)
            net.infer(test.images, out)
            q = torch.empty((len(test.cls), 64, 4), dtype=torch.float64, device=DEV)
            t = torch.empty((len(test.cls), 1, 2), dtype=torch.float64, device=DEV)
            tg3.Cnn.match_propose(out, z, qg_d, 64, 1, 3, q, t)
            torch.cuda.synchronize()
            ang = learned.angle_deg(q.cpu().numpy(), test.quat_true[:, None, :]).min(1)
            return float(np.mean(ang < 10.0))

        before = within10()
        t_star = torch.as_tensor(train.trans_true).to(DEV)
        losses = learned.train_match(net, train.images, refs_train, t_star, train.cls, 2, 256,
                                     2e-3, seed=2)
        after = within10()
    finally:
        net.close()
        ctx.close()
    assert losses[-1] < losses[0]
    assert after > 0.6 and after > before + 0.3, (before, after)
