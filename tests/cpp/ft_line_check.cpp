// Host check of the feature transform's per-line envelope code
// (voxel_ma_gb300/csrc/vc_ft_line.cuh, the same source the device kernel
// runs): random lines of candidates, dense and sparse, with many exact
// ties, against a brute-force lexicographic minimum; small rings force the
// spill and refill paths.  Prints "ok <lines>" or the first mismatch.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "../../voxel_ma_gb300/csrc/vc_ft_line.cuh"

using vc::kFtInf;

template <class I, int RING, int PF>
static bool check_line(const std::vector<int64_t>& in, std::vector<int64_t>& out, std::vector<int32_t>& sm,
                       std::vector<int64_t>& sv) {
    const int L = (int)in.size();
    int32_t rm[RING];
    int64_t rv[RING];
    out.assign(L, -7);
    auto load = [&](int q) { return in[q]; };
    auto emit = [&](int x, int64_t v) {
        if (x < 0 || x >= L || out[x] != -7) {
            std::printf("bad emit at %d\n", x);
            std::exit(2);
        }
        out[x] = v;
    };
    vc::ft_envelope_line<I, RING, PF>(L, load, emit, rm, rv, 1, sm.data(), sv.data(), 1);
    for (int x = 0; x < L; ++x) {
        int64_t best = kFtInf;
        for (int q = 0; q < L; ++q) {
            if (in[q] == kFtInf) continue;
            const int64_t d = x - q;
            const int64_t c = vc::ft_pack(vc::ft_g(in[q]) + d * d, vc::ft_id(in[q]));
            if (c < best) best = c;
        }
        if (out[x] != best) {
            std::printf("mismatch I=%d RING=%d PF=%d L=%d x=%d got (%lld,%d) want (%lld,%d)\n", (int)sizeof(I), RING, PF, L, x,
                        (long long)vc::ft_g(out[x]), vc::ft_id(out[x]), (long long)vc::ft_g(best), vc::ft_id(best));
            return false;
        }
    }
    return true;
}

int main(int argc, char** argv) {
    const int nlines = argc > 1 ? std::atoi(argv[1]) : 20000;
    std::mt19937_64 rng(12345);
    std::vector<int32_t> sm(40000);
    std::vector<int64_t> sv(40000), out;
    for (int it = 0; it < nlines; ++it) {
        const int L = 1 + (int)(rng() % (it % 10 == 0 ? 700 : 70));
        const int mode = (int)(rng() % 6);
        std::vector<int64_t> in(L, kFtInf);
        const int gmax = mode == 0 ? 2 : mode == 1 ? 10 : mode == 2 ? 300 : mode == 3 ? 5000 : 3000000;
        const double p = mode == 4 ? 0.02 : mode == 5 ? 0.3 : 0.9;
        const int idmax = 1 + (int)(rng() % 50);
        for (int q = 0; q < L; ++q) {
            if ((double)(rng() % 1000) / 1000.0 >= p) continue;
            int64_t g = (int64_t)(rng() % (uint64_t)(gmax + 1));
            if (mode == 2) g = g * g % 2000;  // squares: many exact ties
            in[q] = vc::ft_pack(g, (int32_t)(rng() % (uint64_t)idmax));
        }
        // int32 arithmetic covers lines below 2048 points with values below
        // 2^23; int64 covers the rest (and is checked on the same lines)
        bool ok = check_line<int32_t, 8, 8>(in, out, sm, sv) && check_line<int32_t, 2, 8>(in, out, sm, sv) &&
                  check_line<int32_t, 4, 1>(in, out, sm, sv) && check_line<int64_t, 16, 4>(in, out, sm, sv) &&
                  check_line<int64_t, 2, 8>(in, out, sm, sv);
        if (ok && it % 50 == 0) {
            // large values (coordinates up to 2^15): int64 only
            const int L2 = 1 + (int)(rng() % 3000);
            std::vector<int64_t> big(L2, kFtInf);
            for (int q = 0; q < L2; ++q)
                if (rng() % 4 == 0)
                    big[q] = vc::ft_pack((int64_t)(rng() % (1ull << 30)), (int32_t)(rng() % 1000));
            ok = check_line<int64_t, 8, 8>(big, out, sm, sv);
        }
        if (!ok) return 1;
    }
    std::printf("ok %d\n", nlines);
    return 0;
}
