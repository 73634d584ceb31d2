// One lattice line of the feature transform's envelope passes, written once
// for the device kernel (vc_ft.cu) and for a host check of the same code
// against brute force (tests/cpp/ft_line_check.cpp).
//
// Input: for q = 0..L-1 a packed candidate (g << 32 | id) or kFtInf (no
// candidate).  Output: for every x the lexicographic minimum over q of
// ((x - q)^2 + g(q), id(q)), packed the same way (kFtInf when the line has
// no candidate).
//
// The lower envelope of the parabolas is built with a stack; a candidate r
// placed after the top p wins from the smallest integer x given by
// ft_cross_threshold on.  Streaming: after candidate q is placed, point x is
// final once (q + 1 - x)^2 > D(x): every later candidate is at least that
// far away, so none can reach D(x) or tie it.  Final points are emitted at
// once.  An entry whose start lies below the output frontier can never be
// popped (that would beat a final value), so only the entries covering
// [frontier - 1, q] are kept: on dense inputs a few entries, although the
// whole envelope of a line holds most of its points.  The live entries sit
// in a ring of RING slots (shared memory on the device); entries beyond the
// ring spill to global memory and come back when popped down to.
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#include <cmath>
#define VC_HD
#else
#define VC_HD __host__ __device__
#endif

namespace vc {

constexpr int64_t kFtInf = INT64_MAX;

VC_HD inline int64_t ft_pack(int64_t g, int32_t id) { return (g << 32) | (uint32_t)id; }
VC_HD inline int64_t ft_g(int64_t p) { return p >> 32; }
VC_HD inline int32_t ft_id(int64_t p) { return (int32_t)(uint32_t)(p & 0xffffffffLL); }

// Arithmetic of one line in type I: int32_t when every coordinate is below
// 2048 (squared distances then stay below 3 * 2^22 < 2^24, exact in int32
// and in float), int64_t otherwise (coordinates below 2^15).

// Does candidate r (position qr, value gr, index ir) beat candidate p in the
// (value, index) order at x?
template <class I>
VC_HD inline bool ft_beats_at(I x, I qr, I gr, int32_t ir, I qp, I gp, int32_t ip) {
    const I vr = (x - qr) * (x - qr) + gr, vp = (x - qp) * (x - qp) + gp;
    return vr < vp || (vr == vp && ir < ip);
}

// Smallest integer x at which candidate r beats candidate p (position
// qp < qr), clamped to [0, L]: every use compares it with start thresholds
// in [0, L) and with L, and clamping preserves those comparisons.  The
// single-precision quotient is only a first guess: within [-2, L + 2]
// (L < 2^15) its relative error is below 2^-21, so its floor is within one
// of the true floor, which exact integer products then settle.
template <class I>
VC_HD inline int ft_cross_threshold(I qp, I gp, int32_t ip, I qr, I gr, int32_t ir, int L) {
    const I den = 2 * (qr - qp);
    const I num = qr * qr - qp * qp + gr - gp;
#ifdef __CUDA_ARCH__
    const float qf = __fdividef((float)num, (float)den);
#else
    const float qf = (float)num / (float)den;
#endif
    if (qf < -2.0f) return 0;
    if (qf > (float)L + 2.0f) return L;
#ifdef __CUDA_ARCH__
    I fl = (I)floorf(qf);
#else
    I fl = (I)std::floor(qf);
#endif
    if (fl * den > num) --fl;
    else if ((fl + 1) * den <= num) ++fl;
    I t = (fl * den == num && ir < ip) ? fl : fl + 1;
    t = t < 0 ? 0 : (t > (I)L ? (I)L : t);
    return (int)t;
}

// The line: load(q) gives candidate q, emit(x, v) takes the result at x, in
// increasing x.  Ring slot j of this line is ring_meta[j * rs] /
// ring_val[j * rs]; spilled entry k is spill_meta[k * ss] / spill_val[k *
// ss].  PF candidates are loaded ahead of their use.  A candidate is popped
// when the new one beats it at its own start (no division); the new
// candidate's start is the one crossing threshold computed per placement.
// The entry covering the frontier and the value it gives there are kept in
// registers and updated only when a placement reaches the frontier.
template <class I, int RING, int PF, class Load, class Emit>
VC_HD inline void ft_envelope_line(int L, Load load, Emit emit, int32_t* ring_meta, int64_t* ring_val, int64_t rs,
                                   int32_t* spill_meta, int64_t* spill_val, int64_t ss) {
    static_assert((RING & (RING - 1)) == 0, "ring size must be a power of two");
    // live stack: entries [bot, k); [bot, lo) spilled, [lo, k) in the ring
    int k = 0, lo = 0, bot = 0;
    int tq = 0, tz = 0;  // top of stack: position and start threshold
    int64_t tv = 0;      // top of stack: value
    // frontier: points below xf are written; entry cb covers xf, giving it
    // value fd (index fid); the next entry starts at nz (L: none)
    int xf = 0, cb = 0, nz = 0, cq = 0;
    I cg = 0, fd = 0;
    int32_t fid = 0;
    auto meta_of = [&](int j) -> int32_t {
        return j < lo ? spill_meta[(int64_t)j * ss] : ring_meta[(int64_t)(j & (RING - 1)) * rs];
    };
    auto val_of = [&](int j) -> int64_t {
        return j < lo ? spill_val[(int64_t)j * ss] : ring_val[(int64_t)(j & (RING - 1)) * rs];
    };
    int64_t nxt[PF];
#pragma unroll
    for (int u = 0; u < PF; ++u) nxt[u] = u < L ? load(u) : kFtInf;
    for (int q0 = 0; q0 < L; q0 += PF) {
        int64_t cur[PF];
#pragma unroll
        for (int u = 0; u < PF; ++u) {
            cur[u] = nxt[u];
            const int q = q0 + PF + u;
            nxt[u] = q < L ? load(q) : kFtInf;
        }
#pragma unroll
        for (int u = 0; u < PF; ++u) {
            const int q = q0 + u;
            if (q >= L) break;
            const int64_t cv = cur[u];
            if (cv != kFtInf) {
                const I g = (I)ft_g(cv);
                const int32_t id = ft_id(cv);
                // pop every top that the new candidate beats at the top's start
                while (k > 0 && ft_beats_at<I>((I)tz, (I)q, g, id, (I)tq, (I)ft_g(tv), ft_id(tv))) {
                    --k;
                    if (k == 0) {
                        lo = 0;
                        bot = 0;
                        break;
                    }
                    const int64_t j = (int64_t)((k - 1) & (RING - 1)) * rs;
                    if (k - 1 < lo) {  // cached part empty: bring entry k-1 back
                        lo = k - 1;
                        ring_meta[j] = spill_meta[(int64_t)(k - 1) * ss];
                        ring_val[j] = spill_val[(int64_t)(k - 1) * ss];
                    }
                    const int32_t m = ring_meta[j];
                    tv = ring_val[j];
                    tq = m & 0xffff;
                    tz = m >> 16;
                }
                const int thr =
                    k == 0 ? 0 : ft_cross_threshold<I>((I)tq, (I)ft_g(tv), ft_id(tv), (I)q, g, id, L);
                // placed unless it wins only beyond the end of the line (a
                // candidate that popped anything is always placed)
                if (thr < L) {
                    if (lo < bot) lo = bot;  // entries below bot are dead
                    if (k - lo == RING) {    // ring full: spill its bottom entry
                        const int64_t j = (int64_t)(lo & (RING - 1)) * rs;
                        spill_meta[(int64_t)lo * ss] = ring_meta[j];
                        spill_val[(int64_t)lo * ss] = ring_val[j];
                        ++lo;
                    }
                    const int64_t j = (int64_t)(k & (RING - 1)) * rs;
                    ring_meta[j] = q | (thr << 16);
                    ring_val[j] = cv;
                    if (thr <= xf) {  // it covers the frontier now
                        cb = k;
                        cq = q;
                        cg = g;
                        fid = id;
                        const I d = (I)(xf - q);
                        fd = g + d * d;
                        nz = L;
                    } else if (k == cb + 1) {
                        nz = thr;
                    }
                    tq = q;
                    tz = thr;
                    tv = cv;
                    ++k;
                }
            }
            // write the points that are final now
            if (k > 0) {
                const bool last = q + 1 == L;
                while (xf <= q) {
                    const I dn = (I)(q + 1 - xf);
                    if (!last && dn * dn <= fd) break;  // a later candidate may still win here
                    emit(xf, ft_pack((int64_t)fd, fid));
                    bot = cb;
                    ++xf;
                    if (xf == nz) {  // the next entry takes over
                        ++cb;
                        const int32_t m = meta_of(cb);
                        const int64_t v = val_of(cb);
                        cq = m & 0xffff;
                        cg = (I)ft_g(v);
                        fid = ft_id(v);
                        nz = cb + 1 < k ? (meta_of(cb + 1) >> 16) : L;
                    }
                    const I d = (I)(xf - cq);
                    fd = cg + d * d;
                }
            }
        }
    }
    if (k == 0)
        for (int x = 0; x < L; ++x) emit(x, kFtInf);
}

}  // namespace vc
