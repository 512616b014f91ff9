"""Oracle (test infrastructure only): numpy restatement of the learned warm
start's 3D convolutional U-Net, its loss, its gradients and one Adam step.

The network has no counterpart in the reference (whose solves always start
from the previous displacement, src/Solving_CG_GMGS.m:7), so parity is
pinned in two steps:
  * with ``emulate=False`` everything is float64 and ``grad`` is checked
    against central finite differences of ``loss`` (tests/test_oracle_cpu.py);
  * with ``emulate=True`` the device's rounding points are reproduced: BF16
    activations (round to nearest even) after every epilogue, BF16 weights in
    every convolution, FP32 activation gradients rounded to BF16 where they
    are a convolution operand.  The GPU is compared with this form.

Layout and graph follow include/sgld_gpu.h (sgld_net_*): channels-last [v][c]
with v = y + ny (x + nx z); encoder relu(conv3) x2 + 2x average pooling
(ceil, mean over existing children); decoder relu(conv3) on the coarser
level, nearest 2x upsampling plus the skip, relu(conv3); linear 1x1x1 head.
"""
from __future__ import annotations

import numpy as np


def bf16(x):
    """Round to bfloat16 (nearest even) through float32; returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _ident(x):
    return np.asarray(x, dtype=np.float64)


class UNet:
    def __init__(self, dims, cin, cout, levels, widths=None, emulate=True):
        self.cin, self.cout, self.L = int(cin), int(cout), int(levels)
        self.w = list(widths) if widths is not None else [16, 32, 48, 64][: self.L]
        self.dims = [tuple(int(d) for d in dims)]
        for _ in range(1, self.L):
            self.dims.append(tuple((d + 1) // 2 for d in self.dims[-1]))
        self.r = bf16 if emulate else _ident
        self.conv = []   # (cin, cout, taps, level, w_off, b_off)
        off = 0

        def add(ci, co, taps, level):
            nonlocal off
            self.conv.append((ci, co, taps, level, off, off + taps * ci * co))
            off += taps * ci * co + co

        L, w = self.L, self.w
        for l in range(L):
            add(self.cin if l == 0 else w[l - 1], w[l], 27, l)
            add(w[l], w[l], 27, l)
        for l in range(L - 2, -1, -1):
            add(w[l + 1], w[l], 27, l + 1)
            add(w[l], w[l], 27, l)
        add(w[0], self.cout, 1, 0)
        self.nparam = off

    # convolution indices (sgld_net.cu)
    def ca(self, l):
        return 2 * l

    def cb(self, l):
        return 2 * l + 1

    def cu(self, l):
        return 2 * self.L + 2 * (self.L - 2 - l)

    def cm(self, l):
        return 2 * self.L + 2 * (self.L - 2 - l) + 1

    def chead(self):
        return 4 * self.L - 2

    def unpack(self, params):
        p = np.asarray(params, dtype=np.float64)
        out = []
        for ci, co, taps, _, wo, bo in self.conv:
            out.append((p[wo:bo].reshape(taps, ci, co), p[bo:bo + co]))
        return out

    # ---- primitives on [nz, nx, ny, C] grids ----
    def _grid(self, a, level):
        ny, nx, nz = self.dims[level]
        return a.reshape(nz, nx, ny, -1)

    @staticmethod
    def _shifts(taps):
        if taps == 1:
            return [(0, 0, 0)]
        return [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]   # (dz, dx, dy)

    def _conv(self, x, W, b, level):
        """sum_t x[nb(v, t)] @ W[t] (+ b); x [V][ci] (already rounded as the device stages it)."""
        g = self._grid(x, level)
        nz, nx, ny, _ = g.shape
        taps = W.shape[0]
        p = np.pad(g, ((1, 1), (1, 1), (1, 1), (0, 0)))
        out = np.zeros((nz, nx, ny, W.shape[2]))
        for t, (dz, dx, dy) in enumerate(self._shifts(taps)):
            out += p[1 + dz:1 + dz + nz, 1 + dx:1 + dx + nx, 1 + dy:1 + dy + ny] @ W[t]
        out = out.reshape(-1, W.shape[2])
        return out + b if b is not None else out

    def _conv_wgrad(self, x, g, taps, level):
        """dW[t] = sum_v x[nb(v, t)] (x) g[v] and db = sum_v g[v]."""
        xg = self._grid(x, level)
        nz, nx, ny, ci = xg.shape
        p = np.pad(xg, ((1, 1), (1, 1), (1, 1), (0, 0)))
        gg = g.reshape(-1, g.shape[1])
        dW = np.zeros((taps, ci, g.shape[1]))
        for t, (dz, dx, dy) in enumerate(self._shifts(taps)):
            xs = p[1 + dz:1 + dz + nz, 1 + dx:1 + dx + nx, 1 + dy:1 + dy + ny].reshape(-1, ci)
            dW[t] = xs.T @ gg
        return dW, gg.sum(axis=0)

    def _conv_bwd(self, g, W, level):
        """gradient of the input: conv with the spatially flipped, transposed weights."""
        Wt = W[::-1].transpose(0, 2, 1)
        return self._conv(g, Wt, None, level)

    def _pool(self, f, level):
        ny, nx, nz = self.dims[level]
        cy, cx, cz = self.dims[level + 1]
        g = self._grid(f, level)
        s = np.zeros((cz, cx, cy, g.shape[3]))
        n = np.zeros((cz, cx, cy, 1))
        for dz in range(2):
            for dx in range(2):
                for dy in range(2):
                    sub = g[dz::2, dx::2, dy::2]
                    s[:sub.shape[0], :sub.shape[1], :sub.shape[2]] += sub
                    n[:sub.shape[0], :sub.shape[1], :sub.shape[2]] += 1
        return (s / n).reshape(-1, g.shape[3]), n.reshape(-1, 1)

    def _up(self, c, level):
        """nearest 2x upsampling from level+1 to level."""
        ny, nx, nz = self.dims[level]
        g = self._grid(c, level + 1)
        u = g.repeat(2, axis=0).repeat(2, axis=1).repeat(2, axis=2)[:nz, :nx, :ny]
        return u.reshape(-1, g.shape[3])

    def _up_T(self, f, level):
        """transpose of _up: sum over children."""
        cy, cx, cz = self.dims[level + 1]
        g = self._grid(f, level)
        s = np.zeros((cz, cx, cy, g.shape[3]))
        for dz in range(2):
            for dx in range(2):
                for dy in range(2):
                    sub = g[dz::2, dx::2, dy::2]
                    s[:sub.shape[0], :sub.shape[1], :sub.shape[2]] += sub
        return s.reshape(-1, g.shape[3])

    # ---- network ----
    def forward(self, params, x):
        r = self.r
        P = [(r(W), b) for W, b in self.unpack(params)]
        L = self.L
        c = {"X": r(x)}

        def relu_conv(k, inp, level):
            W, b = P[k]
            return r(np.maximum(self._conv(inp, W, b, level), 0.0))

        for l in range(L):
            inp = c["X"] if l == 0 else c[f"P{l}"]
            c[f"Ea{l}"] = relu_conv(self.ca(l), inp, l)
            c[f"E{l}"] = relu_conv(self.cb(l), c[f"Ea{l}"], l)
            if l + 1 < L:
                pooled, cnt = self._pool(c[f"E{l}"], l)
                c[f"P{l + 1}"] = r(pooled)
                c[f"cnt{l + 1}"] = cnt
        prev = c[f"E{L - 1}"]
        for l in range(L - 2, -1, -1):
            c[f"Du{l}"] = relu_conv(self.cu(l), prev, l + 1)
            c[f"S{l}"] = r(self._up(c[f"Du{l}"], l) + c[f"E{l}"])
            c[f"D{l}"] = relu_conv(self.cm(l), c[f"S{l}"], l)
            prev = c[f"D{l}"]
        c["last"] = prev
        W, b = P[self.chead()]
        y = self._conv(prev, W, b, 0)
        c["P"] = P
        return y, c

    @staticmethod
    def loss(y, t, m=None):
        d = y - t
        m = np.ones(y.shape[0]) if m is None else np.asarray(m, float)
        den = y.shape[1] * max(m.sum(), 1e-300)
        return float((m[:, None] * d * d).sum() / den), 2.0 * m[:, None] * d / den

    def backward(self, cache, gy):
        r, P, L = self.r, cache["P"], self.L
        grads = [None] * len(self.conv)

        def wgrad(k, inp, gout, level):
            dW, db = self._conv_wgrad(inp, r(gout), P[k][0].shape[0], level)
            grads[k] = (dW, db)

        def bwd(k, gout, level, mask_act):
            gi = self._conv_bwd(r(gout), P[k][0], level)
            return gi * (mask_act > 0) if mask_act is not None else gi

        last = cache["last"]
        wgrad(self.chead(), last, gy, 0)
        G = {"last": bwd(self.chead(), gy, 0, last)}
        if L > 1:
            G["D0"] = G.pop("last")
        else:
            G["E0"] = G.pop("last")
        for l in range(0, L - 1):
            wgrad(self.cm(l), cache[f"S{l}"], G[f"D{l}"], l)
            gS = bwd(self.cm(l), G[f"D{l}"], l, None)
            G[f"Du{l}"] = self._up_T(gS, l) * (cache[f"Du{l}"] > 0)
            G[f"E{l}"] = gS * (cache[f"E{l}"] > 0)
            pname = f"D{l + 1}" if l + 1 <= L - 2 else f"E{L - 1}"
            wgrad(self.cu(l), cache[pname], G[f"Du{l}"], l + 1)
            G[pname] = bwd(self.cu(l), G[f"Du{l}"], l + 1, cache[pname])
        for l in range(L - 1, -1, -1):
            wgrad(self.cb(l), cache[f"Ea{l}"], G[f"E{l}"], l)
            G[f"Ea{l}"] = bwd(self.cb(l), G[f"E{l}"], l, cache[f"Ea{l}"])
            wgrad(self.ca(l), cache["X"] if l == 0 else cache[f"P{l}"], G[f"Ea{l}"], l)
            if l > 0:
                gP = bwd(self.ca(l), G[f"Ea{l}"], l, None)
                up = self._up(gP / cache[f"cnt{l}"], l - 1)
                G[f"E{l - 1}"] = G[f"E{l - 1}"] + up * (cache[f"E{l - 1}"] > 0)
        flat = np.zeros(self.nparam)
        for (ci, co, taps, _, wo, bo), (dW, db) in zip(self.conv, grads):
            flat[wo:bo] = dW.ravel()
            flat[bo:bo + co] = db
        return flat

    def value_and_grad(self, params, x, t, m=None):
        y, cache = self.forward(params, x)
        loss, gy = self.loss(y, t, m)
        return loss, self.backward(cache, gy), y


def adam_step(w, mom, vel, g, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) with bias correction; returns (w, m, v)."""
    mom = b1 * mom + (1 - b1) * g
    vel = b2 * vel + (1 - b2) * g * g
    c1, c2 = 1.0 / (1 - b1 ** step), 1.0 / (1 - b2 ** step)
    w = w - lr * (mom * c1) / (np.sqrt(vel * c2) + eps)
    return w, mom, vel
