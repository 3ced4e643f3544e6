"""Oracle: the fast autoregressive sampler on the CPU (torch).

Restates deepar/samplers/fast_autoregressive.py:13-76 with
deepar/graph_analysis/dependency_graph.py:35-94: every (layer, site) node of
ConvNetAutoregressive2D is evaluated exactly once, as a [B, taps*Cin] x
[taps*Cin, Cout] product (graph_analysis/convolutional_topology.py:22-30),
after all the sites it depends on are drawn. The evaluation order is one
topological order of that graph: for each site, the head at the site, then
the horizontal stream of every layer at the site; at the end of a row the
vertical stream of every layer over the row. Sites are drawn with the
Philox uniforms of ``oracle.philox`` (+1 iff p(+1) > U).

Used as the CPU baseline of the sampling stage. Test infrastructure only.
"""
import numpy as np
import torch

from . import ar2d, philox


class FastSamplerCPU:
    def __init__(self, params, shape, depth, weights_normalization, dtype=torch.float32):
        self.h, self.w = shape
        self.depth = depth
        self.n_cc = ar2d.num_causal_convs(depth)
        self.dtype = dtype
        p = ar2d.params_to(params, dtype)
        self.k = {}
        for i in range(self.n_cc):
            for c in ar2d.CONV_NAMES:
                name = f"cc{i}.{c}"
                k = ar2d.effective_kernel(p, name, weights_normalization).detach()
                self.k[name] = (k.reshape(-1, k.shape[-1]), p[name + ".bias"].detach())
        self.k["out"] = (p["out.kernel"].reshape(-1, 4), p["out.bias"])
        self.f = p["out.kernel"].shape[2]

    def _taps(self, x, r, c, offsets):
        """Stack x[:, r+dr, c+dc, :] over the taps (zero outside the lattice)."""
        b, ch = x.shape[0], x.shape[-1]
        parts = []
        for dr, dc in offsets:
            rr, cc = r + dr, c + dc
            if 0 <= rr < self.h and 0 <= cc < self.w:
                parts.append(x[:, rr, cc, :])
            else:
                parts.append(torch.zeros((b, ch), dtype=self.dtype))
        return torch.cat(parts, dim=1)

    def sample(self, batch, seed, offset):
        h, w, f, n_cc = self.h, self.w, self.f, self.n_cc
        relu = torch.relu
        z = lambda ch: torch.zeros((batch, h, w, ch), dtype=self.dtype)
        spins = z(1)
        v = [z(f) for _ in range(n_cc)]
        hs = [z(f) for _ in range(n_cc)]
        cat = [z(f) for _ in range(n_cc)]
        tv = [(-2 + i, -1 + j) for i in range(3) for j in range(3)]
        th = [(0, -2 + j) for j in range(3)]
        tc = [(-2 + i, -2 + j) for i in range(3) for j in range(3)]
        u = torch.as_tensor(philox.ar_site_uniforms(seed, offset, batch, h * w), dtype=torch.float64)
        for i in range(n_cc):
            ky, by = self.k[f"cc{i}.y"]
            cat[i][:, 0, :, f // 2:] = relu(by)
        kx, bx = self.k[f"cc{n_cc - 1}.x"]
        cat[n_cc - 1][:, :, 0, :f // 2] = relu(bx)

        def vin(i):
            return spins if i == 0 else v[i - 1]

        def hin(i):
            return spins if i == 0 else hs[i - 1]

        def second(i):
            return i >= 2 and i % 2 == 0 and i != n_cc - 1

        def h_ops(i, r, c):
            kh, bh = self.k[f"cc{i}.h"]
            kx, bx = self.k[f"cc{i}.x"]
            t = relu(self._taps(hin(i), r, c, th) @ kh + bh)
            s = 1 if i == n_cc - 1 else 0
            if c + s < w:
                cat[i][:, r, c + s, :f // 2] = relu(t @ kx + bx)
            if i == n_cc - 1:
                return
            kc, bc = self.k[f"cc{i}.c"]
            hp = self._taps(cat[i], r, c, tc) @ kc + bc
            res = hs[i - 2][:, r, c] if second(i) else 0
            hs[i][:, r, c] = relu(hp + res)

        for r in range(h):
            for c in range(w):
                kc, bc = self.k[f"cc{n_cc - 1}.c"]
                ko, bo = self.k["out"]
                g = relu(self._taps(cat[n_cc - 1], r, c, tc) @ kc + bc)
                l = (g @ ko + bo).to(torch.float64)
                re = l[:, 0:2] - 0.5 * torch.logsumexp(2 * l[:, 0:2], dim=1, keepdim=True)
                up = torch.exp(2 * re[:, 0]) > u[:, r * w + c]
                spins[:, r, c, 0] = torch.where(up, 1.0, -1.0).to(self.dtype)
                for i in range(n_cc):
                    h_ops(i, r, c)
            for i in range(n_cc):
                kv, bv = self.k[f"cc{i}.v"]
                ky, by = self.k[f"cc{i}.y"]
                for c in range(w):
                    vp = self._taps(vin(i), r, c, tv) @ kv + bv
                    if i != n_cc - 1:
                        res = v[i - 2][:, r, c] if second(i) else 0
                        v[i][:, r, c] = relu(vp + res)
                    if r + 1 < h:
                        cat[i][:, r + 1, c, f // 2:] = relu(relu(vp) @ ky + by)
        return spins[..., 0].to(torch.int8).numpy()
