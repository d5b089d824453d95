// hd_tune.cpp -- autotuner for brick shape, persistent-grid size and queue
// schedule.
//
// Replaces the reference's launch-shape choice by the occupancy API
// (getOccupancy, hello.cu:1910-1954), whose data-block y size even follows
// the occupancy result (hello.cu:917).  Here the data layout never depends on
// the GPU; the brick shape (words x rows x planes per warp), the number of
// resident CTAs per SM and the queue schedule (pair order of a batch, mapping
// of queue items to warps) are searched, by timing real runs on the caller's
// pairs.  Winners are kept per workload class and can be persisted
// as a small JSON table.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "hd/hd.h"
#include "hd_internal.h"

namespace hdh {

std::string tune_key(int se, double mean_voxels, int npairs) {
    const int vb = mean_voxels > 1 ? (int)std::lround(std::log2(mean_voxels)) : 0;
    const char* pc = npairs <= 1 ? "p1" : (npairs < 16 ? "p2" : "p16");
    char buf[64];
    std::snprintf(buf, sizeof buf, "se%d/v%d/%s", se == 0 ? 6 : 18, vb, pc);
    return buf;
}

bool TuneTable::save(const std::string& path) const {
    std::ofstream f(path, std::ios::trunc);
    if (!f) return false;
    f << "{\n  \"version\": 1,\n  \"entries\": {";
    bool first = true;
    for (const auto& kv : entries) {
        const Shape& sh = kv.second.shape;
        f << (first ? "\n" : ",\n") << "    \"" << kv.first << "\": {\"kernel\": " << sh.kernel
          << ", \"bxw\": " << sh.bxw << ", \"bz\": " << sh.bz << ", \"steps\": " << sh.steps
          << ", \"ctas_per_sm\": " << sh.ctas_per_sm << ", \"order\": " << sh.order
          << ", \"spread\": " << sh.spread << ", \"us\": " << kv.second.us << "}";
        first = false;
    }
    f << "\n  }\n}\n";
    return (bool)f;
}

// Reads the table written by save(): entries "key": {"bxw": N, "bz": N,
// "ctas_per_sm": N, "us": X}.  Unknown text is skipped.
bool TuneTable::load(const std::string& path) {
    std::ifstream f(path);
    if (!f) return false;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string s = ss.str();
    size_t pos = s.find("\"entries\"");
    if (pos == std::string::npos) return false;
    auto field = [](const std::string& body, const char* name, double* v) {
        const std::string key = std::string("\"") + name + "\"";
        size_t p = body.find(key);
        if (p == std::string::npos) return false;
        p = body.find(':', p);
        if (p == std::string::npos) return false;
        *v = std::strtod(body.c_str() + p + 1, nullptr);
        return true;
    };
    while (true) {
        size_t k0 = s.find('"', pos + 9);
        if (k0 == std::string::npos) break;
        size_t k1 = s.find('"', k0 + 1);
        size_t b0 = s.find('{', k1);
        size_t b1 = s.find('}', b0);
        if (k1 == std::string::npos || b0 == std::string::npos || b1 == std::string::npos) break;
        const std::string key = s.substr(k0 + 1, k1 - k0 - 1);
        const std::string body = s.substr(b0, b1 - b0 + 1);
        double kernel = 1, bxw = 0, bz = 0, steps = 1, cps = 0, order = 0, spread = 0, us = 0;
        if (field(body, "bxw", &bxw) && field(body, "bz", &bz)) {
            field(body, "kernel", &kernel);
            field(body, "steps", &steps);
            field(body, "ctas_per_sm", &cps);
            field(body, "order", &order);
            field(body, "spread", &spread);
            field(body, "us", &us);
            TuneEntry e;
            e.shape.kernel = (int)kernel;
            e.shape.bxw = (int)bxw;
            e.shape.bz = (int)bz;
            e.shape.steps = (int)steps;
            e.shape.ctas_per_sm = (int)cps;
            e.shape.order = order != 0 ? 1 : 0;
            e.shape.spread = spread != 0 ? 1 : 0;
            e.shape.finish();
            e.us = us;
            entries[key] = e;
        }
        pos = b1;
    }
    return true;
}

}  // namespace hdh

using namespace hdh;

extern "C" hd_status hd_autotune(hd_context* ctx, const hd_pair_desc* pairs, int32_t n, int32_t repeats,
                                 char* report, size_t report_len) {
    if (!ctx || !pairs || n <= 0) return HD_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int se = pairs[0].metric == HD_SE6 ? 0 : 1;
    for (int i = 0; i < n; ++i) {
        if (!pairs[i].a || !pairs[i].b || (pairs[i].metric == HD_SE6 ? 0 : 1) != se)
            return set_error(ctx, HD_ERR_BAD_ARG, "autotune: pairs must share one metric");
        const hd_status st = check_dims(ctx, pairs[i].W, pairs[i].H, pairs[i].D);
        if (st != HD_OK) return st;
    }
    DeviceGuard g(ctx->device);
    if (!g.ok) return set_error(ctx, HD_ERR_CUDA, "cannot select device %d", ctx->device);
    std::vector<PairIn> in;
    for (int i = 0; i < n; ++i) {
        PairIn p{pairs[i].a, pairs[i].b, pairs[i].W, pairs[i].H, pairs[i].D, nullptr, nullptr};
        if (!pairs[i].on_device) {
            p.a = zero_copy_ptr(ctx, pairs[i].a);
            p.b = zero_copy_ptr(ctx, pairs[i].b);
            if (!p.a) p.host_a = pairs[i].a;
            if (!p.b) p.host_b = pairs[i].b;
        }
        in.push_back(p);
    }
    repeats = std::max(1, repeats);
    std::vector<hd_result> res(n), ref(n);
    // every field but `iterations` (the barrier count depends on the shape)
    // must agree across candidates; avg_hd bit for bit (NaN included)
    auto differs = [](const hd_result& x, const hd_result& y) {
        return x.hd != y.hd || x.hd_ab != y.hd_ab || x.hd_ba != y.hd_ba || x.hd_robust != y.hd_robust ||
               x.sum_ab != y.sum_ab || x.sum_ba != y.sum_ba || x.n_a != y.n_a || x.n_b != y.n_b ||
               x.n_a_not_b != y.n_a_not_b || x.n_b_not_a != y.n_b_not_a || x.status != y.status ||
               std::memcmp(&x.avg_hd, &y.avg_hd, sizeof(double)) != 0;
    };
    std::string rep;
    bool have_ref = false;
    // Runs one candidate: a warm-up run checked against the first
    // candidate's results, then `repeats` timed runs (host clock around the
    // whole call, which ends with the results on the host); median.
    auto measure = [&](const Shape& c, double* med) -> hd_status {
        RunOpts ro;
        ro.se = se;
        ro.force_shape = true;
        ro.shape = c;
        hd_status st = run_pairs(ctx, in.data(), n, ctx->stream, ro, res.data());
        if (st != HD_OK && st != HD_EMPTY_MASK) return st;
        if (!have_ref) {
            ref = res;
            have_ref = true;
        } else {
            for (int i = 0; i < n; ++i)
                if (differs(res[i], ref[i]))
                    return set_error(ctx, HD_ERR_CUDA,
                                     "autotune: kernel %d shape %dx%dx%d steps %d order %d spread %d gave a different "
                                     "result on pair %d (hd %d/%d/%d sums %llu/%llu, first shape: hd %d/%d/%d sums "
                                     "%llu/%llu)",
                                     c.kernel, c.bxw, c.by, c.bz, c.steps, c.order, c.spread, i, res[i].hd,
                                     res[i].hd_ab, res[i].hd_ba, (unsigned long long)res[i].sum_ab,
                                     (unsigned long long)res[i].sum_ba, ref[i].hd, ref[i].hd_ab, ref[i].hd_ba,
                                     (unsigned long long)ref[i].sum_ab, (unsigned long long)ref[i].sum_ba);
        }
        std::vector<double> t;
        for (int r = 0; r < repeats; ++r) {
            const auto t0 = std::chrono::steady_clock::now();
            st = run_pairs(ctx, in.data(), n, ctx->stream, ro, res.data());
            const auto t1 = std::chrono::steady_clock::now();
            if (st != HD_OK && st != HD_EMPTY_MASK) return st;
            t.push_back(std::chrono::duration<double, std::micro>(t1 - t0).count());
        }
        std::sort(t.begin(), t.end());
        *med = t[t.size() / 2];
        char line[200];
        std::snprintf(line, sizeof line, "kernel=%d bxw=%d by=%d bz=%d steps=%d cps=%d order=%d spread=%d: %.1f us\n",
                      c.kernel, c.bxw, c.by, c.bz, c.steps, c.ctas_per_sm, c.order, c.spread, *med);
        rep += line;
        return HD_OK;
    };
    // Stage 1, kernels and bricks: the one-step kernel over its brick
    // shapes, the blocked kernel over steps per barrier and depth, each at
    // two grid sizes, with the default queue schedule.
    std::vector<Shape> cands;
    for (int bxw : {2, 4, 8})
        for (int bz : {4, 8, 16}) {
            Shape c;
            c.kernel = 1;
            c.bxw = bxw;
            c.bz = bz;
            cands.push_back(c);
        }
    for (int steps : {1, 2, 3, 4, 5})
        for (int bz : {8, 16}) {
            if (steps > 2 && bz != 8) continue;  // compiled: steps 3, 4, 5 with bz 8 only
            Shape c;
            c.kernel = 2;
            c.steps = steps;
            c.bz = bz;
            cands.push_back(c);
        }
    std::vector<std::pair<double, Shape>> scored;
    for (Shape c : cands) {
        for (int cps : {0, 1}) {
            c.ctas_per_sm = cps;
            c.order = c.spread = 0;
            c.finish();
            double med = 0;
            const hd_status st = measure(c, &med);
            if (st != HD_OK) return st;
            scored.emplace_back(med, c);
        }
    }
    // Stage 2, queue schedule on the three fastest: pair order (as given /
    // largest first) x item-to-warp mapping (CTA-major / spread over SMs).
    std::stable_sort(scored.begin(), scored.end(),
                     [](const std::pair<double, Shape>& x, const std::pair<double, Shape>& y) { return x.first < y.first; });
    const size_t top = std::min<size_t>(3, scored.size());
    for (size_t k = 0; k < top; ++k) {
        for (int order : {0, 1})
            for (int spread : {0, 1}) {
                if (!order && !spread) continue;  // measured in stage 1
                if (order && n < 2) continue;     // one pair: nothing to order
                Shape c = scored[k].second;
                c.order = order;
                c.spread = spread;
                double med = 0;
                const hd_status st = measure(c, &med);
                if (st != HD_OK) return st;
                scored.emplace_back(med, c);
            }
    }
    TuneEntry best;
    best.us = 1e300;
    for (const auto& sc : scored)
        if (sc.first < best.us) {
            best.us = sc.first;
            best.shape = sc.second;
        }
    double vox = 0;
    for (const auto& p : in) vox += (double)p.W * p.H * p.D;
    vox /= n;
    const std::string key = tune_key(se, vox, n);
    ctx->tune.entries[key] = best;
    char line[200];
    std::snprintf(line, sizeof line, "best %s: kernel=%d bxw=%d bz=%d steps=%d cps=%d order=%d spread=%d %.1f us\n",
                  key.c_str(), best.shape.kernel, best.shape.bxw, best.shape.bz, best.shape.steps,
                  best.shape.ctas_per_sm, best.shape.order, best.shape.spread, best.us);
    rep += line;
    if (!ctx->tuning_path.empty() && !ctx->tune.save(ctx->tuning_path))
        set_error(ctx, HD_OK, "autotune: could not write %s", ctx->tuning_path.c_str());
    if (report && report_len) {
        std::strncpy(report, rep.c_str(), report_len - 1);
        report[report_len - 1] = 0;
    }
    return HD_OK;
}
