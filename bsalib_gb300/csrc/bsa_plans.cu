// bsa_plans.cu -- tile plans of the split-precision contractions, chosen by the project's
// autotuner (bsalib_gb300/autotune.py) and loaded from a table.
//
// Each tensor-core contraction has a shape choice that trades padding against work per tile:
//   * the Classic form: the E form (one GEMM family over half the grid pairs, bsa_classic_e.cu)
//     or the D1 / D3 form (two families, bsa_mixed.cu) where both apply;
//   * the E form's FRF-table width W (8, 16, 24, or 32 / 48 as two mode halves of 16 / 24):
//     a wider table pads more modes but changes the grid columns per N tile (128 / NMT) and the
//     epilogue's registers;
//   * the D1 / D3 form's width (8, 16, 24, 32, or 64 as two halves of 32);
//   * the Mesher kernel's mode width NMT (a multiple of 8 from the kept modes to 64);
//   * the E form's mode passes: a width of 16 or 24 in one pass or in two of half the modes
//     (half the epilogue's accumulators per pass, fewer register spills, the same MMAs).
// A plan line names a family, a range of kept modes, of K (= components x loaded nodes) and of
// grid points per axis, and the value; the first matching line wins, and a value that does not
// fit the case (narrower than its modes, or not a built width) falls back to the default rule,
// the narrowest width that holds the modes, E form wherever it applies.
//
// Table file: one plan per line, "family nm_lo nm_hi k_lo k_hi nf_lo nf_hi value" with family
// cls_form | cls_e_width | cls_d_width | msh_width | cls_e_split; '#' starts a comment.  Loaded on first use
// from data/tile_plans.txt beside libbsagpu.so (or the file BSA_TILE_PLANS names), or by
// bsa_gpu_loadTilePlans.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"

namespace bsa {

namespace {

struct TilePlan {
    int family, nm_lo, nm_hi, k_lo, k_hi, nf_lo, nf_hi, value;
};

struct PlanTable {
    std::mutex m;
    std::vector<TilePlan> plans;
    bool loaded = false;
    std::string source;
};

PlanTable &table() {
    static PlanTable t;
    return t;
}

int family_id(const char *name) {
    if (!std::strcmp(name, "cls_form")) return BSA_PLAN_CLS_FORM;
    if (!std::strcmp(name, "cls_e_width")) return BSA_PLAN_CLS_E_WIDTH;
    if (!std::strcmp(name, "cls_d_width")) return BSA_PLAN_CLS_D_WIDTH;
    if (!std::strcmp(name, "msh_width")) return BSA_PLAN_MSH_WIDTH;
    if (!std::strcmp(name, "cls_e_split")) return BSA_PLAN_CLS_E_SPLIT;
    return 0;
}

// Parses a table file; returns the number of plans read or -1 (file missing / bad line).
int parse_file(const char *path, std::vector<TilePlan> &out, std::string &err) {
    FILE *fh = std::fopen(path, "r");
    if (!fh) {
        err = std::string("cannot open ") + path;
        return -1;
    }
    char line[512];
    int n = 0, ln = 0;
    while (std::fgets(line, sizeof line, fh)) {
        ++ln;
        char *c = std::strchr(line, '#');
        if (c) *c = 0;
        char fam[64];
        TilePlan p{};
        const int got = std::sscanf(line, "%63s %d %d %d %d %d %d %d", fam, &p.nm_lo, &p.nm_hi, &p.k_lo, &p.k_hi,
                                    &p.nf_lo, &p.nf_hi, &p.value);
        if (got <= 0) continue;  // blank or comment
        p.family = got == 8 ? family_id(fam) : 0;
        if (!p.family) {
            std::fclose(fh);
            err = std::string(path) + ": bad plan on line " + std::to_string(ln);
            return -1;
        }
        out.push_back(p);
        ++n;
    }
    std::fclose(fh);
    return n;
}

// data/tile_plans.txt beside the library (or $BSA_TILE_PLANS); silently empty if absent.
void load_default_locked(PlanTable &t) {
    if (t.loaded) return;
    t.loaded = true;
    std::string path;
    if (const char *env = std::getenv("BSA_TILE_PLANS")) {
        path = env;
    } else {
        Dl_info info;
        if (dladdr((void *)&bsa_gpu_loadTilePlans, &info) && info.dli_fname) {
            path = info.dli_fname;
            const size_t s = path.find_last_of('/');
            path = (s == std::string::npos ? std::string(".") : path.substr(0, s)) + "/data/tile_plans.txt";
        }
    }
    if (path.empty()) return;
    std::vector<TilePlan> v;
    std::string err;
    if (parse_file(path.c_str(), v, err) >= 0) {
        t.plans = v;
        t.source = path;
    }
}

int lookup(int family, int nm, int K, int nf, int dflt) {
    PlanTable &t = table();
    std::lock_guard<std::mutex> lk(t.m);
    load_default_locked(t);
    for (const TilePlan &p : t.plans)
        if (p.family == family && nm >= p.nm_lo && nm <= p.nm_hi && K >= p.k_lo && K <= p.k_hi && nf >= p.nf_lo &&
            nf <= p.nf_hi)
            return p.value;
    return dflt;
}

}  // namespace

int plan_e_width(int nm, int K, int nf) {
    const int d = nm <= 8 ? 8 : nm <= 16 ? 16 : nm <= 24 ? 24 : nm <= 32 ? 32 : 48;
    const int w = lookup(BSA_PLAN_CLS_E_WIDTH, nm, K, nf, d);
    const bool built = w == 8 || w == 16 || w == 24 || w == 32 || w == 48;
    return built && w >= nm ? w : d;
}

int plan_d_width(int nm, int K, int nf) {
    const int d = nm <= 8 ? 8 : nm <= 16 ? 16 : nm <= 24 ? 24 : nm <= 32 ? 32 : 64;
    const int w = lookup(BSA_PLAN_CLS_D_WIDTH, nm, K, nf, d);
    const bool built = w == 8 || w == 16 || w == 24 || w == 32 || w == 64;
    return built && w >= nm ? w : d;
}

bool plan_prefer_e(int nm, int K, int nf) { return lookup(BSA_PLAN_CLS_FORM, nm, K, nf, 1) != 0; }

int plan_e_split(int W, int nm, int K, int nf) {
    if (W == 8) return 1;
    if (W == 32 || W == 48) return 2;
    // GB300 (24-mode building, 257^2 / 1025^2 grids): 24 as 2 x 12 is 2-8 % faster on both grids;
    // 16 as 2 x 8 2.5 % faster on the 1025^2 grid, 7 % slower on the 257^2 one
    const int d = W == 24 ? 2 : (nf > 700 ? 2 : 1);
    const int v = lookup(BSA_PLAN_CLS_E_SPLIT, nm, K, nf, d);
    return v == 1 || v == 2 ? v : d;
}

int plan_msh_width(int nm, int K) {
    const int d = ((nm + 7) / 8) * 8;
    const int w = lookup(BSA_PLAN_MSH_WIDTH, nm, K, 0, d);
    return (w % 8 == 0 && w >= nm && w <= 64) ? w : d;
}

}  // namespace bsa

extern "C" {

int bsa_gpu_setTilePlan(int family, int nm_lo, int nm_hi, int k_lo, int k_hi, int nf_lo, int nf_hi, int value) {
    if (family < BSA_PLAN_CLS_FORM || family > BSA_PLAN_CLS_E_SPLIT || nm_lo > nm_hi || k_lo > k_hi || nf_lo > nf_hi)
        return bsa::eng().fail(BSA_ERR_ARG, "invalid tile plan");
    bsa::PlanTable &t = bsa::table();
    std::lock_guard<std::mutex> lk(t.m);
    bsa::load_default_locked(t);
    // a plan set here takes precedence over the loaded table
    t.plans.insert(t.plans.begin(), bsa::TilePlan{family, nm_lo, nm_hi, k_lo, k_hi, nf_lo, nf_hi, value});
    return BSA_OK;
}

int bsa_gpu_clearTilePlans(void) {
    bsa::PlanTable &t = bsa::table();
    std::lock_guard<std::mutex> lk(t.m);
    t.plans.clear();
    t.loaded = true;  // and do not load the default table again
    t.source.clear();
    return BSA_OK;
}

int bsa_gpu_loadTilePlans(const char *path) {
    bsa::PlanTable &t = bsa::table();
    std::lock_guard<std::mutex> lk(t.m);
    if (!path) {
        t.loaded = false;
        t.plans.clear();
        bsa::load_default_locked(t);
        return BSA_OK;
    }
    std::vector<bsa::TilePlan> v;
    std::string err;
    if (bsa::parse_file(path, v, err) < 0) return bsa::eng().fail(BSA_ERR_ARG, "%s", err.c_str());
    t.plans = v;
    t.loaded = true;
    t.source = path;
    return BSA_OK;
}

int bsa_gpu_getTilePlan(int family, int nm, int K, int nf, int *value) {
    if (!value) return bsa::eng().fail(BSA_ERR_ARG, "null output");
    switch (family) {
    case BSA_PLAN_CLS_FORM: *value = bsa::plan_prefer_e(nm, K, nf) ? 1 : 0; break;
    case BSA_PLAN_CLS_E_WIDTH: *value = bsa::plan_e_width(nm, K, nf); break;
    case BSA_PLAN_CLS_D_WIDTH: *value = bsa::plan_d_width(nm, K, nf); break;
    case BSA_PLAN_MSH_WIDTH: *value = bsa::plan_msh_width(nm, K); break;
    case BSA_PLAN_CLS_E_SPLIT: *value = bsa::plan_e_split(bsa::plan_e_width(nm, K, nf), nm, K, nf); break;
    default: return bsa::eng().fail(BSA_ERR_ARG, "unknown plan family %d", family);
    }
    return BSA_OK;
}

}  // extern "C"
