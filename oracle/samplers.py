"""Oracle: samplers and Markov-chain diagnostics (numpy).

* ``autoregressive_sample`` restates the exact raster-order sampler of
  deepar/samplers/autoregressive.py:29-48 (+1 iff exp(log p(+1)) > U, the
  +-1 variant of samplers/__init__.py:8-14), fed with the Philox uniforms
  of ``oracle.philox.ar_site_uniforms`` so that it reproduces the GPU draw.
* ``metropolis_hastings`` restates samplers/metropolis_hastings.py:15-145
  (Local and Exchange proposals, exp(min(2 dRe log psi, 0)) > U acceptance,
  warm-up and thinning schedule of :46-65).
* ``metropolis_hastings_hamiltonian`` restates metropolis_hastings.py:170-195
  (connections of the operator as proposals, with the n(s)/n(s') factor).
* ``r_hat_and_correlations`` restates metropolis_hastings.py:8-12,67-89.
Test infrastructure only.
"""
import numpy as np

from . import philox


def autoregressive_sample(cond_log_prob_fn, shape, n_samples, seed, offset):
    """cond_log_prob_fn(batch (B,H,W) +-1 with unsampled sites 0) -> (B,H,W,2)
    log-probabilities. One full evaluation per site, as the reference's slow
    sampler does."""
    hh, ww = shape
    u = philox.ar_site_uniforms(seed, offset, n_samples, hh * ww)
    batch = np.zeros((n_samples, hh, ww), dtype=np.float64)
    for k in range(hh * ww):
        i, j = divmod(k, ww)
        lp = cond_log_prob_fn(batch)
        batch[:, i, j] = np.where(np.exp(lp[:, i, j, 0]) > u[:, k], 1.0, -1.0)
    return batch


def propose(kind, chains, words, shape):
    """Candidate configurations for one sweep. chains (C, *shape) +-1."""
    x0, x1, _, x3 = (np.asarray(w, dtype=np.int64) for w in words)
    cand = chains.copy()
    c = np.arange(chains.shape[0])
    if len(shape) == 1:
        (ll,) = shape
        i = x0 % ll
        if kind == "local":
            cand[c, i] *= -1
        else:
            j = (i + (x1 % 3) - 1) % ll
            cand[c, i], cand[c, j] = chains[c, j], chains[c, i]
    else:
        hh, ww = shape
        r, q = x0 % hh, x3 % ww
        if kind == "local":
            cand[c, r, q] *= -1
        else:
            r2 = (r + (x1 % 3) - 1) % hh
            q2 = (q + ((x1 // 3) % 3) - 1) % ww
            cand[c, r, q], cand[c, r2, q2] = chains[c, r2, q2], chains[c, r, q]
    return cand


def accept(log_psi_cand_re, log_psi_re, u):
    d = 2.0 * (log_psi_cand_re - log_psi_re)
    return (d >= 0) | (np.exp(np.minimum(d, 0.0)) > u)


def metropolis_hastings(log_psi_fn, init_chains, kind, samples_per_chain, unused_samples,
                        discard_ratio, seed, sweep_offset=0):
    """Returns (batch (C*S, *shape) chain-major, acceptance ratio, sweeps used)."""
    chains = np.array(init_chains, dtype=np.float64)
    shape = chains.shape[1:]
    n_chains = chains.shape[0]
    lp = np.real(log_psi_fn(chains))
    sweep = sweep_offset
    accepted = 0

    def one_sweep():
        nonlocal chains, lp, sweep, accepted
        words = philox.mh_words(seed, np.arange(n_chains), sweep)
        cand = propose(kind, chains, words, shape)
        lpc = np.real(log_psi_fn(cand))
        if not np.all(np.isfinite(lpc)):
            raise ValueError("candidates log psi has a non-finite element")
        a = accept(lpc, lp, philox.to_uniform(words[2]))
        chains[a] = cand[a]
        lp[a] = lpc[a]
        sweep += 1
        return int(a.sum())

    if discard_ratio > 0:
        for _ in range((samples_per_chain // discard_ratio) * unused_samples):
            one_sweep()
    out = np.empty((n_chains, samples_per_chain) + shape)
    for i in range(samples_per_chain):
        for _ in range(unused_samples + 1):
            accepted += one_sweep()
        out[:, i] = chains
    ratio = accepted / (n_chains * samples_per_chain * (unused_samples + 1))
    return out.reshape((-1,) + shape), ratio, sweep - sweep_offset


def metropolis_hastings_hamiltonian(log_psi_fn, find_conn, init_chains, samples_per_chain, unused_samples,
                                    discard_ratio, seed, sweep_offset=0):
    """samplers/metropolis_hastings.py:170-195: the candidate is a uniformly
    chosen used connection of find_conn (index floor(U * n) in slot order, U
    from word 0 of the Philox counter (chain, sweep, 0x484D), the product
    rounded to float32 as the GPU forms it); acceptance
    exp(2 dRe log psi + log(n(s) / n(s'))) > U with word 2. Schedule as
    ``metropolis_hastings``. Returns (batch chain-major, acceptance ratio)."""
    chains = np.array(init_chains, dtype=np.float64)
    shape = chains.shape[1:]
    n_chains = chains.shape[0]
    lp = np.real(log_psi_fn(chains))
    sweep = sweep_offset
    accepted = 0
    idx = np.arange(n_chains)

    def one_sweep():
        nonlocal chains, lp, sweep
        words = philox.ham_words(seed, idx, sweep)
        conn, _, use = find_conn(chains)
        use = np.asarray(use, dtype=bool)
        n_s = np.maximum(use.sum(axis=0), 1)
        u0 = philox.to_uniform(words[0]).astype(np.float32)
        k = np.floor(u0 * n_s.astype(np.float32)).astype(np.int64)
        k = np.minimum(k, n_s - 1)
        cand = chains.copy()
        for c in range(n_chains):
            slots = np.nonzero(use[:, c])[0]
            if slots.size:
                cand[c] = conn[slots[k[c]], c]
        _, _, use_c = find_conn(cand)
        n_c = np.maximum(np.asarray(use_c, dtype=bool).sum(axis=0), 1)
        lpc = np.real(log_psi_fn(cand))
        d = 2.0 * (lpc - lp) + np.log(n_s / n_c)
        a = (d >= 0) | (np.exp(np.minimum(d, 0.0)) > philox.to_uniform(words[2]))
        chains[a] = cand[a]
        lp[a] = lpc[a]
        sweep += 1
        return int(a.sum())

    if discard_ratio > 0:
        for _ in range((samples_per_chain // discard_ratio) * unused_samples):
            one_sweep()
    out = np.empty((n_chains, samples_per_chain) + shape)
    for i in range(samples_per_chain):
        for _ in range(unused_samples + 1):
            accepted += one_sweep()
        out[:, i] = chains
    ratio = accepted / (n_chains * samples_per_chain * (unused_samples + 1))
    return out.reshape((-1,) + shape), ratio


def sum_correlations(corr):
    """metropolis_hastings.py:8-12: truncate at the first negative pair sum."""
    for i in range(1, corr.shape[0] // 2):
        if corr[2 * i - 1] + corr[2 * i] < 0:
            return corr[:2 * i].sum()
    return corr.sum()


def r_hat_and_correlations(values, n_chains):
    """metropolis_hastings.py:67-89 -> (r_hat, variance, correlations_sum, ess)."""
    values = np.asarray(values, dtype=np.float64)
    b = values.shape[0]
    spc = b // n_chains
    per = values.reshape(n_chains, spc)
    cm = per.mean(axis=1)
    mean = cm.mean()
    between = (spc / (n_chains - 1.0)) * ((cm - mean) ** 2).sum()
    if spc == 1:
        return 1.0, between, 0.0, b
    within = ((per - cm[:, None]) ** 2).sum(axis=1).mean() / (spc - 1)
    var = ((spc - 1) * within + between) / spc
    r_hat = np.sqrt(var / within)
    v = np.zeros(spc - 1)
    for t in range(spc - 1):
        d = per[:, t + 1:] - per[:, :spc - t - 1]
        v[t] = (d * d).mean(axis=1).mean()
    corr = 1 - v / (2 * var)
    cs = sum_correlations(corr)
    return r_hat, var, cs, b / (1 + 2 * cs)
