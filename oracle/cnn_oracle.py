"""CPU oracle of the pose-proposal network (test infrastructure only).

Float64 numpy restatement of the library's network (csrc/tg3_cnn.cu): six
3x3 convolutions (pad 1, bias, ReLU; strides 1, 2, 1, 2, 1, 2) and two dense
layers, the mixture negative log-likelihood of the true pose, and the
analytic gradient of that loss with respect to every parameter.  The
parameter vector holds, layer after layer, the weights (conv [co][ci][3][3],
dense [out][in]) and then the biases, as the library does.

The tests check this oracle's gradients (the pose loss and the matching
loss) against central finite differences (on a reduced network), and the
library's GPU forward, gradients and losses against this oracle.  There is no reference counterpart: the network is an addition
to the E-step (a learned seed for the particle filter's samples).
"""
import numpy as np

# (cin, cout, hin, hout, stride); stride 0: dense
SHAPES = [(1, 32, 64, 64, 1), (32, 32, 64, 32, 2), (32, 64, 32, 32, 1), (64, 64, 32, 16, 2),
          (64, 128, 16, 16, 1), (128, 128, 16, 8, 2), (8192, 256, 1, 1, 0), (256, 68, 1, 1, 0)]
N_COMP = 8


def layout(shapes=SHAPES):
    """[(weight offset, weight shape, bias offset, cout)] per layer, and the total."""
    out, o = [], 0
    for cin, cout, hin, hout, s in shapes:
        wshape = (cout, cin, 3, 3) if s else (cout, cin)
        nw = int(np.prod(wshape))
        out.append((o, wshape, o + nw, cout))
        o += nw + cout
    return out, o


def bf16(x):
    """Round float32 values to the nearest bf16 (ties to even), as float32."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def conv_fwd(x, W, b, s):
    n, ci, h, _ = x.shape
    ho = h // s
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    y = np.broadcast_to(b[None, :, None, None], (n, W.shape[0], ho, ho)).copy()
    for ky in range(3):
        for kx in range(3):
            xs = xp[:, :, ky:ky + s * ho:s, kx:kx + s * ho:s]
            y += np.einsum("nchw,oc->nohw", xs, W[:, :, ky, kx], optimize=True)
    return y


def conv_bwd(x, W, gy, s):
    n, ci, h, _ = x.shape
    ho = gy.shape[2]
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    gW = np.zeros_like(W)
    gxp = np.zeros_like(xp)
    for ky in range(3):
        for kx in range(3):
            xs = xp[:, :, ky:ky + s * ho:s, kx:kx + s * ho:s]
            gW[:, :, ky, kx] = np.einsum("nohw,nchw->oc", gy, xs, optimize=True)
            gxp[:, :, ky:ky + s * ho:s, kx:kx + s * ho:s] += np.einsum(
                "nohw,oc->nchw", gy, W[:, :, ky, kx], optimize=True)
    return gxp[:, :, 1:-1, 1:-1], gW, gy.sum((0, 2, 3))


def _gram_schmidt(a1, a2):
    n1 = np.linalg.norm(a1, axis=-1, keepdims=True) + 1e-12
    b1 = a1 / n1
    u2 = a2 - (b1 * a2).sum(-1, keepdims=True) * b1
    n2 = np.linalg.norm(u2, axis=-1, keepdims=True) + 1e-12
    b2 = u2 / n2
    return b1, b2, np.cross(b1, b2), n1, n2


def head_loss(out, Rstar, tstar):
    """Per-image loss and its gradient with respect to the outputs.
    out [n][68]; Rstar [n][3][3]; tstar [n][2]."""
    out = np.asarray(out, dtype=np.float64)
    n = out.shape[0]
    comp = out[:, :64].reshape(n, N_COMP, 8)
    r1, r2, r3 = Rstar[:, :, 0][:, None], Rstar[:, :, 1][:, None], Rstar[:, :, 2][:, None]
    a1, a2 = comp[..., 0:3], comp[..., 3:6]
    b1, b2, b3, n1, n2 = _gram_schmidt(a1, a2)
    c = 0.5 * ((b1 * r1).sum(-1) + (b2 * r2).sum(-1) + (b3 * r3).sum(-1) - 1.0)
    raw = comp[..., 6]
    kap = np.where(raw > 20, raw, np.log1p(np.exp(np.minimum(raw, 20)))) + 1e-3
    logit = comp[..., 7]
    llse = logit.max(1, keepdims=True) + np.log(np.exp(logit - logit.max(1, keepdims=True)).sum(1, keepdims=True))
    lp = logit - llse + 1.5 * np.log(kap) + kap * (c - 1.0)
    m = lp.max(1, keepdims=True)
    lse = m + np.log(np.exp(lp - m).sum(1, keepdims=True))
    loss = -lse[:, 0]
    resp = np.exp(lp - lse)
    sm = np.exp(logit - llse)
    g = np.zeros_like(out)
    gc = g[:, :64].reshape(n, N_COMP, 8)
    gc[..., 7] = sm - resp
    sig = np.where(raw > 20, 1.0, 1.0 / (1.0 + np.exp(-np.minimum(raw, 20))))
    gc[..., 6] = -resp * (1.5 / kap + c - 1.0) * sig
    w = (-resp * kap)[..., None]
    gb1 = 0.5 * w * (r1 + np.cross(b2, r3))
    gb2 = 0.5 * w * (r2 + np.cross(r3, b1))
    gu2 = (gb2 - b2 * (b2 * gb2).sum(-1, keepdims=True)) / n2
    ga2 = gu2 - b1 * (b1 * gu2).sum(-1, keepdims=True)
    gb1 = gb1 - (gu2 * (b1 * a2).sum(-1, keepdims=True) + a2 * (b1 * gu2).sum(-1, keepdims=True))
    ga1 = (gb1 - b1 * (b1 * gb1).sum(-1, keepdims=True)) / n1
    gc[..., 0:3] = ga1
    gc[..., 3:6] = ga2
    mu, lv = out[:, 64:66], out[:, 66:68]
    diff = tstar - mu
    e = np.exp(-lv)
    loss = loss + 0.5 * (diff * diff * e + lv).sum(1)
    g[:, 64:66] = -diff * e
    g[:, 66:68] = 0.5 * (1.0 - diff * diff * e)
    g[:, :64] = gc.reshape(n, 64)
    return loss, g


def forward(params, img, shapes=SHAPES, round_bf16=True, round_act=False):
    """Activations of every layer (post-ReLU, the last without).  round_act:
    the image and every hidden layer's output rounded to bf16, as the
    inference forward stores them (tg3_cnn_infer)."""
    lay, _ = layout(shapes)
    x = np.asarray(img, dtype=np.float64).reshape(len(img), 1, shapes[0][2], shapes[0][2])
    if round_act:
        x = bf16(x).astype(np.float64)
    acts = [x]
    for li, ((wo, ws, bo, co), (cin, cout, hin, hout, s)) in enumerate(zip(lay, shapes)):
        W = np.asarray(params[wo:wo + int(np.prod(ws))], dtype=np.float32)
        W = (bf16(W) if round_bf16 else W).astype(np.float64).reshape(ws)
        b = np.asarray(params[bo:bo + co], dtype=np.float64)
        if s:
            y = conv_fwd(acts[-1], W, b, s)
        else:
            y = acts[-1].reshape(len(img), -1) @ W.T + b
        if li < len(shapes) - 1:
            y = np.maximum(y, 0.0)
            if round_act:
                y = bf16(y).astype(np.float64)
        acts.append(y)
    return acts


def loss_and_grad(params, img, Rstar, tstar, shapes=SHAPES, round_bf16=True):
    """Mean loss over the batch and its gradient (the parameter layout)."""
    acts = forward(params, img, shapes, round_bf16)
    loss, g = head_loss(acts[-1], Rstar, tstar)
    return float(loss.mean()), grad_from_output(params, img, g / len(img), shapes, round_bf16,
                                                acts)


def contrastive(out_p, out_r, tstar, tau):
    """Matching loss of n particles' outputs against their n references'
    outputs and its gradient with respect to both: symmetric InfoNCE on the
    cosine similarities / tau of the normalised embeddings (outputs 0..63;
    particle i's positive is reference i) plus the Gaussian shift loss of the
    particles' outputs 64..67 against tstar.  Returns (mean loss, g_p, g_r)."""
    P = np.asarray(out_p, dtype=np.float64)
    Rr = np.asarray(out_r, dtype=np.float64)
    n = len(P)
    u, v = P[:, :64], Rr[:, :64]
    fu = 1.0 / np.sqrt((u * u).sum(1, keepdims=True) + 1e-12)
    fv = 1.0 / np.sqrt((v * v).sum(1, keepdims=True) + 1e-12)
    zp, zr = u * fu, v * fv
    S = zp @ zr.T / tau
    rm = S.max(1, keepdims=True)
    rowL = rm[:, 0] + np.log(np.exp(S - rm).sum(1))
    cm = S.max(0, keepdims=True)
    colL = cm[0] + np.log(np.exp(S - cm).sum(0))
    d = np.diag(S)
    mu, lv = P[:, 64:66], P[:, 66:68]
    diff = tstar - mu
    e = np.exp(-lv)
    loss = 0.5 * (rowL - d) + 0.5 * (colL - d) + 0.5 * (diff * diff * e + lv).sum(1)
    eye = np.eye(n)
    G = (0.5 / n) * ((np.exp(S - rowL[:, None]) - eye) + (np.exp(S - colL[None, :]) - eye))
    dzp = G @ zr / tau
    dzr = G.T @ zp / tau

    def through_norm(x, f, dz):
        # z = x f, f = (|x|^2 + eps)^-1/2:  dL/dx = f dz - f^3 x (x . dz)
        return f * dz - f ** 3 * x * (x * dz).sum(1, keepdims=True)

    g_p = np.zeros_like(P)
    g_r = np.zeros_like(Rr)
    g_p[:, :64] = through_norm(u, fu, dzp)
    g_r[:, :64] = through_norm(v, fv, dzr)
    g_p[:, 64:66] = -diff * e / n
    g_p[:, 66:68] = 0.5 * (1.0 - diff * diff * e) / n
    return float(loss.mean()), g_p, g_r


def grad_from_output(params, img, gout, shapes=SHAPES, round_bf16=True, acts=None):
    """Gradient (the parameter layout) of a loss whose derivative with
    respect to the outputs is gout [n][68]."""
    lay, total = layout(shapes)
    if acts is None:
        acts = forward(params, img, shapes, round_bf16)
    n = len(img)
    grad = np.zeros(total)
    gy = np.asarray(gout, dtype=np.float64)
    for li in range(len(shapes) - 1, -1, -1):
        (wo, ws, bo, co), (cin, cout, hin, hout, s) = lay[li], shapes[li]
        W = np.asarray(params[wo:wo + int(np.prod(ws))], dtype=np.float32)
        W = (bf16(W) if round_bf16 else W).astype(np.float64).reshape(ws)
        if li < len(shapes) - 1:
            gy = gy * (acts[li + 1] > 0)
        if s:
            gx, gW, gb = conv_bwd(acts[li], W, gy, s)
        else:
            xin = acts[li].reshape(n, -1)
            gW = gy.T @ xin
            gb = gy.sum(0)
            gx = (gy @ W).reshape(acts[li].shape)
        grad[wo:wo + gW.size] = gW.ravel()
        grad[bo:bo + co] = gb
        gy = gx
    return grad
