"""Host logic of the pose network's training loop (tg3/learned.py
train_match) on the CPU, with a stand-in network object: the learning-rate
schedule (linear warm-up, then cosine decay) and the first-epoch stall guard
that makes the caller restart from another initialisation."""
import math

import numpy as np
import pytest
import torch

from tg3 import learned


class _Net:
    """The calls train_match makes, recording the learning rates; the loss
    of each batch comes from `loss(k)`."""
    N_OUT = 4

    def __init__(self, loss):
        self.loss, self.k, self.lrs = loss, 0, []

    def forward(self, x, out):
        out.zero_()

    def zero_grads(self):
        pass

    def contrastive(self, outP, outR, tstar, tau, dP, dR):
        v = self.loss(self.k)
        self.k += 1
        return v

    def backward(self, x, d):
        pass

    def adam(self, lr):
        self.lrs.append(lr)


def _data(n=800, classes=2):
    images = torch.zeros((n, 64, 64))
    refs = torch.zeros((n, 64, 64))
    tstar = torch.zeros((n, 2))
    cls = np.arange(n) % classes
    return images, refs, tstar, cls


def test_learning_rate_warms_up_then_decays():
    images, refs, tstar, cls = _data()
    net = _Net(lambda k: 3.0 / (1 + 0.01 * k))
    lr, epochs, batch = 1e-3, 2, 8
    losses = learned.train_match(net, images, refs, tstar, cls, epochs, batch, lr,
                                 warmup=0.1, stall_check=True)
    steps = epochs * (len(cls) // batch)
    warm = int(0.1 * steps)
    assert len(losses) == epochs and len(net.lrs) == steps
    exp = [lr * min(1.0, (k + 1) / warm) * 0.5 * (1 + math.cos(math.pi * k / steps))
           for k in range(steps)]
    np.testing.assert_allclose(net.lrs, exp, rtol=1e-12)
    assert np.argmax(net.lrs) in (warm - 1, warm)
    assert all(a >= b for a, b in zip(net.lrs[warm:], net.lrs[warm + 1:]))


def test_first_epoch_on_the_plateau_raises_training_stalled():
    images, refs, tstar, cls = _data()
    net = _Net(lambda k: 2.98 + 1e-3 * math.sin(k))
    with pytest.raises(learned.TrainingStalled):
        learned.train_match(net, images, refs, tstar, cls, 3, 8, 1e-3, stall_check=True)
    assert net.k == len(cls) // 8          # stopped after the first epoch
    # without the check the same run completes
    net2 = _Net(lambda k: 2.98)
    assert len(learned.train_match(net2, images, refs, tstar, cls, 2, 8, 1e-3)) == 2
