// autotune.cu — autotuner of the wavefront form (crg_autotune_batch).
//
// Coordinate descent from the defaults over the knobs that change speed but
// not results: BVH width {2, 4, 8} (scenes rebuilt with their own build
// options), each scene's leaf size {1, 2, 3} (a large displaced mesh renders
// ~9% faster with one triangle per leaf slot, the 36-triangle box ~8% slower),
// stage fusion {split, shadow-in-shade, one kernel per bounce},
// per-lane refill {off, 4, 8, 16, 24}, warp fetch {32, 64}, block size {128, 256}
// path pool {32M, 64M, 128M} (128M-sample chunks).  Each candidate renders a reduced copy of the
// batch (spp scaled to a sample budget) into scratch films: one untimed run,
// then one run timed with CUDA events on the caller's stream.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "crg_internal.h"

namespace crg {
namespace {

constexpr uint32_t kOff = 0xFFFFFFFFu;

std::string shape_key(crg_scene *const *scenes, uint32_t nscenes, const crg_view *views, uint32_t nviews,
                      const crg_autotune_opts &o) {
    std::string k;
    char buf[96];
    std::snprintf(buf, sizeof buf, "b%llu w%u l%u|", (unsigned long long)o.sample_budget, o.widths, o.leaves);
    k += buf;
    for (uint32_t i = 0; i < nscenes; ++i) {
        // a tuned leaf size is part of the result, not of the batch's shape
        std::snprintf(buf, sizeof buf, "s%u/%u/%u|", scenes[i]->ntri, scenes[i]->opts.treelet,
                      o.leaves ? 0u : scenes[i]->opts.leaf_max);
        k += buf;
    }
    for (uint32_t v = 0; v < nviews; ++v) {
        const crg_settings &s = views[v].settings;
        std::snprintf(buf, sizeof buf, "v%u:%ux%ux%u/%u/%u/%u|", views[v].scene, s.width, s.height, s.spp, s.max_bounces,
                      s.rr_depth, s.mode);
        k += buf;
    }
    return k;
}

struct Trial {
    crg_wavefront_opts o;
    uint32_t width;
    float ms;
};

} // namespace
} // namespace crg

using namespace crg;

extern "C" crg_status crg_autotune_batch(crg_scene *const *scenes, uint32_t nscenes, const crg_view *views, uint32_t nviews,
                                         const crg_autotune_opts *opts, crg_wavefront_opts *best, uint32_t *best_width,
                                         crg_autotune_trial *trials, uint32_t trials_cap, uint32_t *ntrials,
                                         crg_stream stream) {
    if (!scenes || nscenes == 0 || !scenes[0] || !views || nviews == 0 || !best || !best_width) return CRG_ERR_INVALID_ARG;
    crg_context *ctx = scenes[0]->ctx;
    crg_autotune_opts o{};
    if (opts) o = *opts;
    if (o.sample_budget == 0) o.sample_budget = 1ull << 27;
    if (o.widths & ~14u) return set_error(ctx, CRG_ERR_INVALID_ARG, "autotune: widths is a mask of 2 | 4 | 8");
    if (o.leaves & ~14u) return set_error(ctx, CRG_ERR_INVALID_ARG, "autotune: leaves is a mask of 1<<1 | 1<<2 | 1<<3");
    for (uint32_t i = 0; i < nscenes; ++i)
        if (!scenes[i] || scenes[i]->ctx != ctx || !scenes[i]->built)
            return set_error(ctx, CRG_ERR_INVALID_ARG, "autotune: scenes must be built and share one context");
    if (ntrials) *ntrials = 0;
    const std::string key = shape_key(scenes, nscenes, views, nviews, o);
    if (o.reuse) {
        auto it = ctx->tune_cache.find(key);
        if (it != ctx->tune_cache.end()) {
            const uint32_t w = it->second.width;
            for (uint32_t i = 0; i < nscenes; ++i) {
                const uint32_t leaf = i < it->second.leaf.size() ? it->second.leaf[i] : scenes[i]->opts.leaf_max;
                if (scenes[i]->width != w || scenes[i]->opts.leaf_max != leaf) {
                    crg_build_opts bo = scenes[i]->opts;
                    bo.width = w;
                    bo.leaf_max = leaf;
                    const crg_status rc = crg_scene_build(scenes[i], &bo, stream);
                    if (rc != CRG_OK) return rc;
                }
            }
            *best = it->second.opts;
            *best_width = w;
            return CRG_OK;
        }
    }
    cudaStream_t st = (cudaStream_t)stream;
    // reduced batch: spp scaled to the budget, scratch films
    unsigned long long total = 0;
    for (uint32_t v = 0; v < nviews; ++v)
        total += (unsigned long long)views[v].settings.width * views[v].settings.height * views[v].settings.spp;
    if (total == 0) return set_error(ctx, CRG_ERR_INVALID_ARG, "autotune: empty batch");
    const double scale = std::min(1.0, (double)o.sample_budget / (double)total);
    std::vector<crg_view> tv(views, views + nviews);
    std::vector<crg_film *> films(nviews, nullptr);
    unsigned long long trial_samples = 0;
    crg_status rc = CRG_OK;
    for (uint32_t v = 0; v < nviews && rc == CRG_OK; ++v) {
        crg_settings &s = tv[v].settings;
        s.spp = std::max<uint32_t>(1u, (uint32_t)((double)s.spp * scale));
        trial_samples += (unsigned long long)s.width * s.height * s.spp;
        rc = crg_film_create(ctx, s.width, s.height, 0, &films[v]);
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (rc == CRG_OK && cudaEventCreate(&e0) != cudaSuccess) rc = set_error(ctx, CRG_ERR_CUDA, "cudaEventCreate");
    if (rc == CRG_OK && cudaEventCreate(&e1) != cudaSuccess) rc = set_error(ctx, CRG_ERR_CUDA, "cudaEventCreate");

    std::vector<Trial> log;
    auto rebuild = [&](uint32_t w) -> crg_status {
        for (uint32_t i = 0; i < nscenes; ++i) {
            if (scenes[i]->width == w) continue;
            crg_build_opts bo = scenes[i]->opts;
            bo.width = w;
            const crg_status r = crg_scene_build(scenes[i], &bo, stream);
            if (r != CRG_OK) return r;
        }
        return CRG_OK;
    };
    // one candidate: untimed run, then a timed run; returns ms (negative on error)
    auto measure = [&](const crg_wavefront_opts &c, uint32_t width) -> float {
        for (int rep = 0; rep < 2; ++rep) {
            for (uint32_t v = 0; v < nviews; ++v) crg_film_reset(films[v], stream);
            if (rep == 1) cudaEventRecord(e0, st);
            const crg_status r = crg_render_batch(scenes, nscenes, tv.data(), films.data(), nviews, &c, stream);
            if (r != CRG_OK) {
                rc = r;
                return -1.0f;
            }
            if (rep == 1) cudaEventRecord(e1, st);
        }
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        log.push_back(Trial{c, width, ms});
        return ms;
    };

    crg_wavefront_opts cur{1u << 27, 1u << 27, 128, 32, 0, 0, 0, 1, 16};
    uint32_t width = scenes[0]->width;
    float best_ms = -1.0f;
    if (rc == CRG_OK) best_ms = measure(cur, width);
    // BVH width
    if (rc == CRG_OK && o.widths) {
        for (uint32_t w : {2u, 4u, 8u}) {
            if (!(o.widths & w) || w == width || rc != CRG_OK) continue;
            const uint32_t prev = width;
            if ((rc = rebuild(w)) != CRG_OK) break;
            const float ms = measure(cur, w);
            if (rc != CRG_OK) break;
            if (ms < best_ms) {
                best_ms = ms;
                width = w;
            } else if ((rc = rebuild(prev)) != CRG_OK) {
                break;
            }
        }
    }
    // leaf size, one scene at a time
    if (rc == CRG_OK && o.leaves) {
        for (uint32_t i = 0; i < nscenes && rc == CRG_OK; ++i) {
            const uint32_t keep_leaf = scenes[i]->opts.leaf_max;
            uint32_t best_leaf = keep_leaf;
            for (uint32_t leaf = 1; leaf <= 3 && rc == CRG_OK; ++leaf) {
                if (!(o.leaves & (1u << leaf)) || leaf == keep_leaf) continue;
                crg_build_opts bo = scenes[i]->opts;
                bo.leaf_max = leaf;
                if ((rc = crg_scene_build(scenes[i], &bo, stream)) != CRG_OK) break;
                const float ms = measure(cur, width);
                if (rc != CRG_OK) break;
                if (ms < best_ms) {
                    best_ms = ms;
                    best_leaf = leaf;
                }
            }
            if (rc == CRG_OK && scenes[i]->opts.leaf_max != best_leaf) {
                crg_build_opts bo = scenes[i]->opts;
                bo.leaf_max = best_leaf;
                rc = crg_scene_build(scenes[i], &bo, stream);
            }
        }
    }
    // the remaining knobs, one at a time
    auto sweep = [&](auto set, std::initializer_list<uint32_t> values) {
        if (rc != CRG_OK) return;
        crg_wavefront_opts keep = cur;
        for (uint32_t val : values) {
            crg_wavefront_opts c = keep;
            set(c, val);
            if (std::memcmp(&c, &keep, sizeof c) == 0) continue;
            const float ms = measure(c, width);
            if (rc != CRG_OK) return;
            if (ms < best_ms) {
                best_ms = ms;
                cur = c;
            }
        }
    };
    sweep([](crg_wavefront_opts &c, uint32_t v) { c.fuse = v; }, {1u, 2u, 3u});
    if (cur.fuse <= 2) sweep([](crg_wavefront_opts &c, uint32_t v) { c.refill = v; }, {kOff, 4u, 8u, 16u, 24u});
    sweep([](crg_wavefront_opts &c, uint32_t v) { c.fetch = v; }, {32u, 64u});
    sweep([](crg_wavefront_opts &c, uint32_t v) { c.block_size = v; }, {128u, 256u});
    // Path pool, up to the 128M-sample chunk: on a GB300 the 64-view batch renders faster with more paths
    // in flight (32M -> 64M -> 128M paths: +12%, +9%; fewer, fuller iterations), while pools small enough
    // to keep the path state (about 156 B per path) in L2 measured 35-45% slower.  Larger chunks are not
    // searched: a reduced trial batch fits in one of them and rewards them (256M paths in 512M-sample
    // chunks won the trials at 1203 Msamples/s but rendered the full batch at 1110 against 1192).
    sweep([](crg_wavefront_opts &c, uint32_t v) { c.path_pool = v; }, {1u << 25, 1u << 26, 1u << 27});

    for (crg_film *f : films)
        if (f) crg_film_destroy(f);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (rc != CRG_OK) return rc;
    *best = cur;
    *best_width = width;
    std::vector<uint32_t> leaf(nscenes);
    for (uint32_t i = 0; i < nscenes; ++i) leaf[i] = scenes[i]->opts.leaf_max;
    ctx->tune_cache[key] = crg_context::Tuned{cur, width, leaf};
    const uint32_t n = (uint32_t)log.size();
    if (ntrials) *ntrials = n;
    if (trials)
        for (uint32_t i = 0; i < n && i < trials_cap; ++i) {
            trials[i].opts = log[i].o;
            trials[i].width = log[i].width;
            trials[i].ms = log[i].ms;
            trials[i].msamples_per_s = (float)((double)trial_samples / ((double)log[i].ms * 1e3));
            trials[i].pad_ = 0;
        }
    return CRG_OK;
}

namespace {

// "name|sm_count" of the context's device, spaces kept out of the line format
std::string device_tag(crg_context *ctx) {
    cudaDeviceProp p{};
    if (cudaGetDeviceProperties(&p, ctx->device) != cudaSuccess) {
        (void)cudaGetLastError();
        return "unknown|0";
    }
    std::string name(p.name);
    for (char &c : name)
        if (c == ' ' || c == '\t' || c == '\n' || c == '|') c = '_';
    return name + "|" + std::to_string(p.multiProcessorCount);
}

constexpr const char *kCacheHeader = "crg-autotune-cache 1";

} // namespace

extern "C" crg_status crg_autotune_cache_save(crg_context *ctx, const char *path) {
    if (!ctx || !path) return set_error(ctx, CRG_ERR_INVALID_ARG, "autotune cache: null argument");
    std::FILE *f = std::fopen(path, "w");
    if (!f) return set_error(ctx, CRG_ERR_INVALID_ARG, std::string("autotune cache: cannot write ") + path);
    bool ok = std::fprintf(f, "%s\ndevice %s\n", kCacheHeader, device_tag(ctx).c_str()) > 0;
    for (const auto &kv : ctx->tune_cache) {
        const crg_wavefront_opts &o = kv.second.opts;
        ok = ok && std::fprintf(f, "%s\t%u\t%u %u %u %u %u %u %u %u %u\t", kv.first.c_str(), kv.second.width, o.path_pool,
                                o.chunk_samples, o.block_size, o.fetch, o.max_iterations, o.count_work, o.host_loop,
                                o.fuse, o.refill) > 0;
        for (size_t i = 0; i < kv.second.leaf.size(); ++i)
            ok = ok && std::fprintf(f, i ? ",%u" : "%u", kv.second.leaf[i]) > 0;
        ok = ok && std::fputc('\n', f) != EOF;
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return set_error(ctx, CRG_ERR_INVALID_ARG, std::string("autotune cache: write failed: ") + path);
    return CRG_OK;
}

extern "C" crg_status crg_autotune_cache_load(crg_context *ctx, const char *path, uint32_t *count) {
    if (count) *count = 0;
    if (!ctx || !path) return set_error(ctx, CRG_ERR_INVALID_ARG, "autotune cache: null argument");
    std::FILE *f = std::fopen(path, "r");
    if (!f) return set_error(ctx, CRG_ERR_INVALID_ARG, std::string("autotune cache: cannot open ") + path);
    std::vector<std::string> lines;
    {
        std::string cur;
        int ch;
        while ((ch = std::fgetc(f)) != EOF) {
            if (ch == '\n') {
                lines.push_back(cur);
                cur.clear();
            } else {
                cur.push_back((char)ch);
            }
        }
        if (!cur.empty()) lines.push_back(cur);
        std::fclose(f);
    }
    auto bad = [&](size_t line) {
        return set_error(ctx, CRG_ERR_INVALID_ARG,
                         std::string("autotune cache: malformed line ") + std::to_string(line + 1) + " of " + path);
    };
    if (lines.size() < 2 || lines[0] != kCacheHeader) return bad(0);
    if (lines[1].compare(0, 7, "device ") != 0) return bad(1);
    if (lines[1].substr(7) != device_tag(ctx)) return CRG_OK; // measured on another kind of device
    std::vector<std::pair<std::string, crg_context::Tuned>> got;
    for (size_t i = 2; i < lines.size(); ++i) {
        const std::string &l = lines[i];
        if (l.empty()) continue;
        const size_t t1 = l.find('\t');
        const size_t t2 = t1 == std::string::npos ? t1 : l.find('\t', t1 + 1);
        const size_t t3 = t2 == std::string::npos ? t2 : l.find('\t', t2 + 1);
        if (t3 == std::string::npos || t1 == 0) return bad(i);
        crg_context::Tuned tu{};
        crg_wavefront_opts &o = tu.opts;
        char tail = 0;
        if (std::sscanf(l.substr(t1 + 1, t2 - t1 - 1).c_str(), "%u%c", &tu.width, &tail) != 1) return bad(i);
        if (!(tu.width == 2 || tu.width == 4 || tu.width == 8)) return bad(i);
        if (std::sscanf(l.substr(t2 + 1, t3 - t2 - 1).c_str(), "%u %u %u %u %u %u %u %u %u%c", &o.path_pool,
                        &o.chunk_samples, &o.block_size, &o.fetch, &o.max_iterations, &o.count_work, &o.host_loop,
                        &o.fuse, &o.refill, &tail) != 9)
            return bad(i);
        const std::string leaves = l.substr(t3 + 1);
        size_t p = 0;
        while (p < leaves.size()) {
            size_t q = leaves.find(',', p);
            if (q == std::string::npos) q = leaves.size();
            unsigned v = 0;
            if (q == p || std::sscanf(leaves.substr(p, q - p).c_str(), "%u%c", &v, &tail) != 1 || v < 1 || v > 3)
                return bad(i);
            tu.leaf.push_back(v);
            p = q + 1;
        }
        got.emplace_back(l.substr(0, t1), tu);
    }
    for (auto &kv : got) ctx->tune_cache[kv.first] = kv.second;
    if (count) *count = (uint32_t)got.size();
    return CRG_OK;
}
