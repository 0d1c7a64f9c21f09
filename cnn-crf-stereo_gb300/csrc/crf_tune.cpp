// crf_tune.cpp -- the CRF tile table (no counterpart in the reference, whose
// solver has one fixed launch shape).
//
// A tile is the chain kernel's prefetch ring depth and chains per CTA, for
// the H and the V pass separately.  Which tile is fastest depends on the
// label count D (the ring's share of shared memory), the chain lengths W and
// H and the number of chains in flight (pairs per launch); every tile gives
// the same bits.  The table maps (W, H, D, npairs, delta) to the tile that
// cnncrf_batch_autotune / cnncrf_crf_autotune measured fastest, plus the
// times they measured; every solve looks its shape up here and takes the
// default tile (ring 8, 2 chains per CTA) for a shape the table lacks.  The
// table is process-wide and guarded by a mutex; it can be saved to and merged
// from a text file so a deployment tunes once:
//
//   cnncrf-crf-tiles 1
//   # W H D npairs delta ring_h chains_h ring_v chains_v ms_h ms_v
//   1242 375 128 4 3 4 2 4 2 1.0312 0.7154
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/cnncrf.h"
#include "common.h"
#include "kernels.h"

using namespace cnncrf;

namespace {

using Key = std::tuple<int, int, int, int, int>; // W, H, D, npairs, delta

struct Entry {
    k::CrfTile tile;
    float ms_h = 0, ms_v = 0;
};

std::mutex g_mu;
std::map<Key, Entry> g_table;

const char *kMagic = "cnncrf-crf-tiles 1";

bool shape_ok(int W, int H, int D, int np, int delta)
{
    return W >= 1 && H >= 1 && D >= 1 && D <= 256 && np >= 1 && delta >= 1 && delta <= 4;
}

} // namespace

namespace cnncrf {
namespace k {

bool crf_tile_valid(const CrfTile &t)
{
    auto ring = [](int r) { return r == 4 || r == 8; };
    auto wpb = [](int w) { return w == 1 || w == 2 || w == 4; };
    return ring(t.ring_h) && ring(t.ring_v) && wpb(t.wpb_h) && wpb(t.wpb_v);
}

CrfTile crf_tile_lookup(int W, int H, int D, int np, int delta)
{
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_table.find(Key(W, H, D, np, delta));
    return it == g_table.end() ? CrfTile() : it->second.tile;
}

void crf_tile_store(int W, int H, int D, int np, int delta, const CrfTile &t, float ms_h, float ms_v)
{
    std::lock_guard<std::mutex> g(g_mu);
    g_table[Key(W, H, D, np, delta)] = Entry{t, ms_h, ms_v};
}

} // namespace k
} // namespace cnncrf

extern "C" {

int cnncrf_crf_tuning_set(int width, int height, int depth, int npairs, int delta, const cnncrf_crf_tile *tile)
{
    clear_error();
    if (!tile) return fail(CNNCRF_EINVAL, "crf tuning: null tile");
    if (!shape_ok(width, height, depth, npairs, delta))
        return fail(CNNCRF_EINVAL, "crf tuning: bad shape %dx%dx%d x%d delta %d", width, height, depth, npairs, delta);
    k::CrfTile t;
    t.ring_h = tile->ring_h, t.wpb_h = tile->chains_per_cta_h;
    t.ring_v = tile->ring_v, t.wpb_v = tile->chains_per_cta_v;
    if (!k::crf_tile_valid(t))
        return fail(CNNCRF_EINVAL, "crf tuning: ring %d/%d (4 or 8), chains per CTA %d/%d (1, 2 or 4)", t.ring_h,
                    t.ring_v, t.wpb_h, t.wpb_v);
    k::crf_tile_store(width, height, depth, npairs, delta, t, 0.0f, 0.0f);
    return CNNCRF_OK;
}

int cnncrf_crf_tuning_get(int width, int height, int depth, int npairs, int delta, cnncrf_crf_tile *tile,
                          int *found, float *ms_h, float *ms_v)
{
    clear_error();
    if (!tile || !found) return fail(CNNCRF_EINVAL, "crf tuning: null argument");
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_table.find(Key(width, height, depth, npairs, delta));
    const Entry e = it == g_table.end() ? Entry() : it->second;
    *found = it != g_table.end();
    tile->ring_h = e.tile.ring_h, tile->chains_per_cta_h = e.tile.wpb_h;
    tile->ring_v = e.tile.ring_v, tile->chains_per_cta_v = e.tile.wpb_v;
    if (ms_h) *ms_h = e.ms_h;
    if (ms_v) *ms_v = e.ms_v;
    return CNNCRF_OK;
}

int cnncrf_crf_tuning_clear(void)
{
    std::lock_guard<std::mutex> g(g_mu);
    g_table.clear();
    return CNNCRF_OK;
}

int cnncrf_crf_tuning_count(int *n)
{
    if (!n) return fail(CNNCRF_EINVAL, "crf tuning: null argument");
    std::lock_guard<std::mutex> g(g_mu);
    *n = (int)g_table.size();
    return CNNCRF_OK;
}

int cnncrf_crf_tuning_save(const char *path)
{
    clear_error();
    if (!path) return fail(CNNCRF_EINVAL, "crf tuning: null path");
    std::lock_guard<std::mutex> g(g_mu);
    FILE *f = std::fopen(path, "w");
    if (!f) return fail(CNNCRF_EINVAL, "crf tuning: cannot write %s", path);
    std::fprintf(f, "%s\n# W H D npairs delta ring_h chains_h ring_v chains_v ms_h ms_v\n", kMagic);
    for (const auto &kv : g_table) {
        const Key &key = kv.first;
        const Entry &e = kv.second;
        std::fprintf(f, "%d %d %d %d %d %d %d %d %d %.4f %.4f\n", std::get<0>(key), std::get<1>(key),
                     std::get<2>(key), std::get<3>(key), std::get<4>(key), e.tile.ring_h, e.tile.wpb_h, e.tile.ring_v,
                     e.tile.wpb_v, e.ms_h, e.ms_v);
    }
    const bool ok = std::fclose(f) == 0;
    return ok ? CNNCRF_OK : fail(CNNCRF_EINVAL, "crf tuning: cannot write %s", path);
}

// Reads the whole file first: a malformed file changes nothing.
int cnncrf_crf_tuning_load(const char *path)
{
    clear_error();
    if (!path) return fail(CNNCRF_EINVAL, "crf tuning: null path");
    FILE *f = std::fopen(path, "r");
    if (!f) return fail(CNNCRF_EINVAL, "crf tuning: cannot read %s", path);
    std::vector<std::pair<Key, Entry>> rows;
    char line[512];
    int lineno = 0, rc = CNNCRF_OK;
    while (rc == CNNCRF_OK && std::fgets(line, sizeof line, f)) {
        ++lineno;
        std::string s(line);
        while (!s.empty() && (s.back() == '\n' || s.back() == '\r' || s.back() == ' ')) s.pop_back();
        if (lineno == 1) {
            if (s != kMagic) rc = fail(CNNCRF_EINVAL, "crf tuning: %s: first line is not '%s'", path, kMagic);
            continue;
        }
        size_t p = s.find_first_not_of(" \t");
        if (p == std::string::npos || s[p] == '#') continue;
        int W, H, D, np, dl;
        Entry e;
        char extra;
        const int got = std::sscanf(s.c_str(), "%d %d %d %d %d %d %d %d %d %f %f %c", &W, &H, &D, &np, &dl,
                                    &e.tile.ring_h, &e.tile.wpb_h, &e.tile.ring_v, &e.tile.wpb_v, &e.ms_h, &e.ms_v,
                                    &extra);
        if (got != 11 || !shape_ok(W, H, D, np, dl) || !k::crf_tile_valid(e.tile))
            rc = fail(CNNCRF_EINVAL, "crf tuning: %s line %d: '%s'", path, lineno, s.c_str());
        else
            rows.push_back({Key(W, H, D, np, dl), e});
    }
    std::fclose(f);
    if (rc == CNNCRF_OK && lineno == 0) rc = fail(CNNCRF_EINVAL, "crf tuning: %s is empty", path);
    if (rc != CNNCRF_OK) return rc;
    std::lock_guard<std::mutex> g(g_mu);
    for (auto &r : rows) g_table[r.first] = r.second;
    return CNNCRF_OK;
}

} // extern "C"
