"""Restatement, in numpy, of the device's own draw rules (device-drawn mode).

TEST INFRASTRUCTURE ONLY: tests compare the CUDA selection stage against these
functions, and rebuild the event tape of a device-drawn generation from them so
that the oracle can replay it.  The product path never imports this module.

Parent sampling, the breakpoint and strand-swap draws of every gamete, the
per-row mutation counts and the new alleles' positions are restated bit for
bit; allele effects (Box-Muller through the device's log and cos) only to a
few FP64 ulps.  What is restated, and from where:
  * the fitness-proportional rule itself is the reference's
    SelectionGenerator::update (include/clotho/data_spaces/selection/
    general_fitness_selection_generator.hpp:45-69): uniform parents when every
    fitness is equal, else a parent with probability fitness / total.  The
    reference draws through Boost's discrete_distribution; the engine draws one
    uniform per parent and searches an inclusive prefix sum of fitness for the
    first entry above u * total (upper_bound), which is the same law;
  * the random stream is the engine's own (no reference counterpart):
    Philox-4x32-10 from its published description (Salmon, Moraes, Dror, Shaw,
    "Parallel random numbers: as easy as 1, 2, 3", SC'11), keyed by the
    population seed, counter (offspring index, 0, generation, stream 2);
    uniforms are the top 53 bits of two 32-bit outputs times 2^-53;
  * breakpoints: E ~ Poisson(rho) per gamete by CDF inversion (the reference's
    crossover_event_distribution_helper.hpp:25-36 draws Poisson(rho) too),
    positions uniform in [0, 1) (position_distribution_helper.hpp:27-41), the
    swap bit Bernoulli(bias) (batch_crossover_mtwe.hpp:135-145); new mutations
    Poisson(mu) per offspring row, which sums to the reference's
    M ~ Poisson(2N mu) with uniform target rows (mutation_allocator.hpp:41-47,
    batch_mutation_task_population_space_row.hpp:77);
  * the FP64 prefix sum follows the device scan's association order exactly
    (chunks of 4,096 entries, 1,024 threads of four entries each, a
    Hillis-Steele scan inside each 32-lane warp, sequential sums across warps
    and across chunks), so the prefix sums and the total are bit-identical to
    the device's, and so are the sampled parents.
"""
from __future__ import annotations

import numpy as np

_MASK = np.uint64(0xFFFFFFFF)
STREAM_GAMETE, STREAM_SELECT, STREAM_MUT_COUNT, STREAM_MUT_ALLELE = 1, 2, 3, 4


def philox4x32(c0, c1, c2, c3, key: int):
    """Philox-4x32-10 over arrays of 32-bit counters; returns four uint64 arrays of 32-bit words."""
    c = [np.asarray(x, dtype=np.uint64) & _MASK for x in (c0, c1, c2, c3)]
    shape = np.broadcast(*c).shape
    c0, c1, c2, c3 = (np.broadcast_to(x, shape).copy() for x in c)
    k0 = np.uint64(key & 0xFFFFFFFF)
    k1 = np.uint64((key >> 32) & 0xFFFFFFFF)
    m0, m1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
    w0, w1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
    for _ in range(10):
        p0 = m0 * c0  # < 2^64: exact
        p1 = m1 * c2
        n0 = (p1 >> np.uint64(32)) ^ c1 ^ k0
        n2 = (p0 >> np.uint64(32)) ^ c3 ^ k1
        c0, c1, c2, c3 = n0, p1 & _MASK, n2, p0 & _MASK
        k0 = (k0 + w0) & _MASK
        k1 = (k1 + w1) & _MASK
    return c0, c1, c2, c3


def u01(hi, lo) -> np.ndarray:
    """[0, 1) double from the top 53 of 64 random bits (exact: v < 2^53)."""
    v = ((np.asarray(hi, np.uint64) << np.uint64(32)) | np.asarray(lo, np.uint64)) >> np.uint64(11)
    return v.astype(np.float64) * 2.0 ** -53


def fitness_prefix(fit) -> tuple[np.ndarray, float, bool]:
    """(inclusive prefix sums, total, all-equal) of the device's three-phase FP64 scan."""
    fit = np.ascontiguousarray(fit, np.float64)
    N = fit.size
    if N == 0:
        return np.zeros(0), 0.0, True
    chunk = 4096
    nch = (N + chunk - 1) // chunk
    v = np.zeros(nch * chunk)
    v[:N] = fit
    v = v.reshape(nch, 32, 32, 4)           # chunk, warp, lane, element
    s = ((v[..., 0] + v[..., 1]) + v[..., 2]) + v[..., 3]   # thread sums (0.0 + v0 == v0)
    x = s.copy()
    for o in (1, 2, 4, 8, 16):               # warp inclusive scan, Hillis-Steele
        y = x[..., :-o].copy()
        x[..., o:] = x[..., o:] + y
    sw = x[..., 31]                           # warp totals [nch, 32]
    t = np.zeros(nch)
    woff = np.zeros((nch, 32))
    for i in range(32):                       # sequential across warps
        woff[:, i] = t
        t = t + sw[:, i]
    part = np.zeros(nch)
    acc = 0.0
    for c in range(nch):                      # sequential across chunks
        part[c] = acc
        acc = acc + t[c]
    excl = np.zeros_like(x)
    excl[..., 1:] = x[..., :-1]
    r = part[:, None, None] + (woff[:, :, None] + excl)
    out = np.empty_like(v)
    for k in range(4):
        r = r + v[..., k]
        out[..., k] = r
    cdf = out.reshape(-1)[:N].copy()
    same = bool(np.all(fit == fit[0]))
    return cdf, float(acc), same


def select_parents(parent_fit, N: int, gen: int, seed: int):
    """Parents of N offspring (2N entries, (id0, id1) per offspring) drawn as the
    device draws them from the parents' fitness; also returns whether the draw
    was uniform and the prefix sums."""
    parent_fit = np.ascontiguousarray(parent_fit, np.float64)
    Np = parent_fit.size
    cdf, total, same = fitness_prefix(parent_fit)
    k = np.arange(N, dtype=np.uint64)
    x0, x1, x2, x3 = philox4x32(k, 0, gen, STREAM_SELECT, seed)
    u = np.stack([u01(x0, x1), u01(x2, x3)], axis=1)        # [N, 2]
    uniform = same or not (total > 0.0)
    if Np == 0:
        ids = np.zeros((N, 2), np.int64)
    elif uniform:
        ids = np.minimum(np.floor(u * float(Np)).astype(np.int64), Np - 1)
    else:
        target = u * total
        ids = np.minimum(np.searchsorted(cdf, target, side="right"), Np - 1)
    return ids.reshape(-1).astype(np.uint32), uniform, cdf, total


def poisson_inv(u, lam: float, e: float) -> np.ndarray:
    """Poisson draw by sequential inversion of the CDF, as the device computes it:
    p_0 = F_0 = e = exp(-lam) (from the host's C library), then
    p_k = p_{k-1} * (lam * (1/k)), F_k = F_{k-1} + p_k, each operation rounded
    separately; the draw is the first k with u <= F_k (k <= 4096)."""
    u = np.asarray(u, np.float64)
    k = np.zeros(u.shape, np.int64)
    p = np.full(u.shape, e)
    F = np.full(u.shape, e)
    live = u > F
    step = 0
    while live.any() and step < 4096:
        step += 1
        p = np.where(live, p * (lam * (1.0 / step)), p)
        F = np.where(live, F + p, F)
        k = np.where(live, step, k)
        live = live & (u > F)
    return k


def gamete_draws(S: int, gen: int, seed: int, rho: float, bias: float, q1: bool, exp_neg_rho: float,
                 max_events: int = 128):
    """Per-gamete breakpoint counts, strand-swap bits and breakpoint positions of a
    device-drawn generation: counter (gamete, 0, generation, stream 1) gives the count
    (Poisson(rho) by inversion) and the swap bit (u < bias); counter
    (gamete, 1 + k/2, ...) gives breakpoints k (even k: first two words, odd k: last
    two).  Under the reference's crossover rule (Q1) odd gametes draw no breakpoint."""
    g = np.arange(S, dtype=np.uint64)
    x0, x1, x2, x3 = philox4x32(g, 0, gen, STREAM_GAMETE, seed)
    E = poisson_inv(u01(x0, x1), rho, exp_neg_rho)
    swap = (u01(x2, x3) < bias).astype(np.uint8)
    if q1:
        E[1::2] = 0
    E = np.minimum(E, max_events)
    ev_off = np.zeros(S + 1, np.uint32)
    ev_off[1:] = np.cumsum(E)
    ev_pos = np.zeros(int(ev_off[-1]), np.float64)
    kmax = int(E.max()) if S else 0
    for k in range(kmax):
        rows = np.nonzero(E > k)[0]
        a0, a1, a2, a3 = philox4x32(rows.astype(np.uint64), 1 + (k >> 1), gen, STREAM_GAMETE, seed)
        ev_pos[ev_off[rows] + k] = u01(a0, a1) if (k & 1) == 0 else u01(a2, a3)
    return E, swap, ev_off, ev_pos


def mutation_draws(S: int, gen: int, seed: int, mu: float, exp_neg_mu: float):
    """New mutations of a device-drawn generation: Poisson(mu) per offspring row from
    counter (row, 0, generation, stream 3); mutations are numbered row by row (the
    exclusive prefix of the counts), and mutation i's position is the uniform of
    counter (i, 0, generation, stream 4).  Returns (target row per mutation, positions)."""
    r = np.arange(S, dtype=np.uint64)
    x0, x1, _, _ = philox4x32(r, 0, gen, STREAM_MUT_COUNT, seed)
    cnt = poisson_inv(u01(x0, x1), mu, exp_neg_mu)
    mut_seq = np.repeat(np.arange(S, dtype=np.uint32), cnt)
    i = np.arange(mut_seq.size, dtype=np.uint64)
    y0, y1, _, _ = philox4x32(i, 0, gen, STREAM_MUT_ALLELE, seed)
    return mut_seq, u01(y0, y1)


def mutation_effects(M: int, T: int, gen: int, seed: int, p_neutral: float, eff_mean: float, eff_sigma: float):
    """Allele effects of mutations 0..M-1 by the device's rule (FP64, before rounding to
    FP32): trait t of mutation i is neutral (0) iff the uniform of counter
    (i, 1 + t, generation, stream 4) is below p_neutral, else mean + sigma * n with n a
    Box-Muller normal from u1 = 1 - (the same counter's second uniform) and u2 from
    counter (i, 5 + t, ...): n = sqrt(-2 ln u1) cos(2 pi u2).  numpy's log and cos
    stand in for the device's, so values agree to a few FP64 ulps, not bit for bit."""
    out = np.zeros((M, T), np.float64)
    i = np.arange(M, dtype=np.uint64)
    for t in range(T):
        a0, a1, a2, a3 = philox4x32(i, 1 + t, gen, STREAM_MUT_ALLELE, seed)
        b0, b1, _, _ = philox4x32(i, 5 + t, gen, STREAM_MUT_ALLELE, seed)
        live = ~(u01(a0, a1) < p_neutral)
        u1 = 1.0 - u01(a2, a3)
        u2 = u01(b0, b1)
        n = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
        out[:, t] = np.where(live, eff_mean + eff_sigma * n, 0.0)
    return out
