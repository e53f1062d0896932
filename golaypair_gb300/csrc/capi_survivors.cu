// capi_survivors.cu -- generation output options: the file format switch,
// the text exporter of binary survivor files (format in survivors.h), and
// the spectral pruning switch (its lookup table).
#include <cstdio>
#include <string>
#include <vector>

#include "ctx.h"
#include "survivors.h"

namespace {

bool read_all(const char* path, std::string& out) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    out.clear();
    char buf[1 << 16];
    size_t got;
    while ((got = fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, got);
    const bool ok = !ferror(f);
    fclose(f);
    return ok;
}

int fail_or(gp_ctx* c, int code, const char* what, const char* path) {
    return c ? c->fail(code, "%s: %s", what, path) : code;
}

}  // namespace

extern "C" {

int gp_set_output_format(gp_ctx* c, int format) {
    if (!c) return GP_ERR_ARG;
    if (format != GP_FORMAT_TEXT && format != GP_FORMAT_BINARY)
        return c->fail(GP_ERR_ARG, "unknown output format %d", format);
    c->out_format = format;
    return GP_OK;
}

int gp_set_spectral_prune(gp_ctx* c, int on) {
    if (!c) return GP_ERR_ARG;
    if (on && !c->prune_tab.p) {
        // m <= kPruneTab - 1: squares, and norms x^2 + xy + y^2 (x, y >= 0;
        // the same set as a^2 - ab + b^2 over all integers)
        std::vector<uint8_t> tab(kPruneTab, 0);
        for (int x = 0; x * x < kPruneTab; ++x) tab[x * x] |= 1;
        for (int x = 0; x * x < kPruneTab; ++x)
            for (int y = 0; y <= x && x * x + x * y + y * y < kPruneTab; ++y) tab[x * x + x * y + y * y] |= 2;
        cudaSetDevice(c->device);
        if (!c->prune_tab.ensure(kPruneTab)) return c->fail(GP_ERR_NOMEM, "spectral prune table");
        GP_CUDA_TRY(c, cudaMemcpy(c->prune_tab.p, tab.data(), kPruneTab, cudaMemcpyHostToDevice));
    }
    c->spectral_prune = on ? 1 : 0;
    return GP_OK;
}

int gp_export_text(gp_ctx* c, const char* in_path, const char* out_path) {
    if (!in_path || !out_path) return c ? c->fail(GP_ERR_ARG, "export: null path") : GP_ERR_ARG;
    std::string bytes;
    if (!read_all(in_path, bytes)) return fail_or(c, GP_ERR_IO, "export: cannot read", in_path);
    gp::SurvHeader h;
    const uint8_t* body = nullptr;
    if (gp::surv_parse(bytes, h, &body) != 1) return fail_or(c, GP_ERR_FORMAT, "export: not a survivor file", in_path);
    std::string text;
    if (!gp::surv_to_text(h, body, text)) return fail_or(c, GP_ERR_FORMAT, "export: malformed record in", in_path);
    FILE* f = fopen(out_path, "wb");
    if (!f) return fail_or(c, GP_ERR_IO, "export: cannot write", out_path);
    bool ok = text.empty() || fwrite(text.data(), 1, text.size(), f) == text.size();
    ok = (fclose(f) == 0) && ok;
    return ok ? GP_OK : fail_or(c, GP_ERR_IO, "export: write failed", out_path);
}

}  // extern "C"
