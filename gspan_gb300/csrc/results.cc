// Result collector: every emitted pattern appended to one flat int32 buffer,
// so a caller (a Python binding, say) takes a run's results in one copy
// instead of one callback per pattern.
#include "gspan_gb300.h"

#include <new>
#include <vector>

struct gspan_results {
    std::vector<int32_t> words;
    int64_t patterns = 0;
};

extern "C" {

gspan_results* gspan_results_create(void) { return new (std::nothrow) gspan_results(); }

void gspan_results_destroy(gspan_results* r) { delete r; }

void gspan_results_clear(gspan_results* r)
{
    if (!r) return;
    r->words.clear();
    r->patterns = 0;
}

int gspan_results_batch_emit(void* user, int32_t instance, const gspan_pattern_edge* code, int32_t len,
                             int32_t support)
{
    gspan_results* r = static_cast<gspan_results*>(user);
    if (!r || len < 0) return 1;
    try {
        r->words.push_back(instance);
        r->words.push_back(len);
        r->words.push_back(support);
        for (int32_t i = 0; i < len; ++i) {
            r->words.push_back(code[i].from);
            r->words.push_back(code[i].to);
            r->words.push_back(code[i].from_label);
            r->words.push_back(code[i].edge_label);
            r->words.push_back(code[i].to_label);
        }
    } catch (const std::bad_alloc&) {
        return 1;   // stops mining: GSPAN_ERR_ABORTED
    }
    ++r->patterns;
    return 0;
}

int gspan_results_emit(void* user, const gspan_pattern_edge* code, int32_t len, int32_t support)
{
    return gspan_results_batch_emit(user, 0, code, len, support);
}

int64_t gspan_results_patterns(const gspan_results* r) { return r ? r->patterns : 0; }

const int32_t* gspan_results_data(const gspan_results* r, int64_t* nwords)
{
    if (nwords) *nwords = r ? (int64_t)r->words.size() : 0;
    return r && !r->words.empty() ? r->words.data() : nullptr;
}

}  // extern "C"
