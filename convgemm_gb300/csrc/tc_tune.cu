// Per-shape tile configuration chosen by the autotuner (convgemm_gb300/autotune.py):
// the output-channel width of a tile (64 / 128 / 256) for the forward and
// input-gradient kernels, and the tile width and pixel-split count of the
// weight gradient.  Shapes without an entry use the built-in heuristics.
#include <array>
#include <map>
#include <mutex>

#include "../../include/convgemm_gpu.h"
#include "tc_host.h"

namespace {

using Key = std::array<int, 14>;
std::mutex g_tune_mu;
std::map<Key, TcTune> g_tune;

Key key_of(int op, const convgemm_shape_t &s) {
    return {op, s.b, s.h, s.w, s.c, s.kn, s.kh, s.kw, s.vpad, s.hpad, s.vstride, s.hstride, s.vdil, s.hdil};
}

}  // namespace

bool tc_tune_get(int op, const convgemm_shape_t &s, TcTune *t) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key_of(op, s));
    if (it == g_tune.end()) return false;
    *t = it->second;
    return true;
}

extern "C" convgemm_status_t convgemm_tune_set(int op, const convgemm_shape_t *shape, int bn, int splits) {
    if (!shape || op < CONVGEMM_TUNE_FWD || op > CONVGEMM_TUNE_FWD_BF16X3)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_tune_set: bad operation or NULL shape");
    if (bn != 0 && bn != 64 && bn != 128 && bn != 256)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_tune_set: tile width %d is not 0/64/128/256", bn);
    const bool mt_op = op == CONVGEMM_TUNE_FWD || op == CONVGEMM_TUNE_DGRAD;
    // forward / input gradient: M tiles per weight tile (1 / 2) + 4 for eight epilogue warps
    // weight gradient: pixel splits in bits 0-15, CONVGEMM_WGRAD_* flags above
    const bool aux_ok = op == CONVGEMM_TUNE_WGRAD ? (splits >= 0 && (splits & ~0x3fbffff) == 0)
                        : mt_op ? ((splits & ~24) == 0 || (splits & ~24) == 1 || (splits & ~24) == 2 ||
                                   (splits & ~24) == 5 || (splits & ~24) == 6)
                                : splits == 0;
    if (!aux_ok)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE,
                            "convgemm_tune_set: aux is the weight gradient's split count (plus CONVGEMM_WGRAD_* flags), or for the BF16 forward / "
                            "input gradient 1 / 2 M tiles per weight tile, plus 4 for eight epilogue warps, plus 8 for the general "
                            "kernel instead of the slab kernel, plus 16 for one K block per ring stage");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    if (bn == 0 && splits == 0)
        g_tune.erase(key_of(op, *shape));
    else
        g_tune[key_of(op, *shape)] = TcTune{bn, splits};
    return CONVGEMM_SUCCESS;
}

extern "C" void convgemm_tune_clear(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
}
