// Binary checkpoint / restart of a context (the reference has none).
//
// A context's device state is one arena whose layout is a pure function of
// its particle counts, cell grid and form, so a checkpoint is a fixed header
// followed by the arena's raw bytes: restoring it into a context created with
// the same parameters and form continues the run bit-identically (state, cell
// lists of both buffers, neighbour lists, list stamps, error record).  A
// context with the same counts, grid and form but other physical parameters
// (a restart with a new time step, say) may load it too.
//
// Layout (little-endian, as the host writes it):
//   offset 0   char[8]   "SPHNJCK1"
//          8   uint32    header bytes (sizeof CkHeader)
//         12   uint32    form
//         16   int32     step, parity, virt_sorted, virt_cells_valid
//         32   uint64    arena bytes
//         40   sphnj_params (verbatim, sizeof reported by sphnj_abi_sizeof(0))
//   then the arena.
#include "context.h"

#include <cstdio>
#include <cstring>
#include <vector>

using namespace sphnj;

namespace {

struct CkHeader {
    char magic[8];
    uint32_t header_bytes;
    uint32_t form;
    int32_t step, parity, virt_sorted, virt_cells_valid;
    uint64_t arena_bytes;
    sphnj_params params;
};

const char kMagic[8] = {'S', 'P', 'H', 'N', 'J', 'C', 'K', '1'};

int ck_fail(sphnj_ctx *c, int code, const char *m) {
    if (c) c->msg = m;
    return code;
}

int ck_cuda(sphnj_ctx *c, cudaError_t e, const char *where) {
    if (c) c->msg = std::string(where) + ": " + cudaGetErrorString(e);
    return SPHNJ_ERR_CUDA;
}

CkHeader header_of(const sphnj_ctx *ctx) {
    CkHeader h;
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, kMagic, 8);
    h.header_bytes = sizeof(CkHeader);
    h.form = (uint32_t)ctx->form;
    h.step = ctx->step;
    h.parity = ctx->parity;
    h.virt_sorted = ctx->virt_sorted ? 1 : 0;
    h.virt_cells_valid = ctx->virt_cells_valid ? 1 : 0;
    h.arena_bytes = ctx->arena_bytes;
    h.params = ctx->p;
    return h;
}

}  // namespace

extern "C" {

int sphnj_checkpoint_size(const sphnj_ctx *ctx, uint64_t *bytes) {
    if (!ctx || !bytes) return SPHNJ_ERR_ARG;
    *bytes = sizeof(CkHeader) + ctx->arena_bytes;
    return SPHNJ_OK;
}

int sphnj_checkpoint_save(sphnj_ctx *ctx, void *buffer, uint64_t bytes) {
    if (!ctx || !buffer) return SPHNJ_ERR_ARG;
    if (!ctx->uploaded) return ck_fail(ctx, SPHNJ_ERR_ARG, "checkpoint before sphnj_upload");
    if (bytes < sizeof(CkHeader) + ctx->arena_bytes) return ck_fail(ctx, SPHNJ_ERR_ARG, "checkpoint buffer too small");
    cudaSetDevice(ctx->device);
    const CkHeader h = header_of(ctx);
    std::memcpy(buffer, &h, sizeof h);
    cudaError_t e = cudaMemcpyAsync(static_cast<char *>(buffer) + sizeof h, ctx->arena, ctx->arena_bytes,
                                    cudaMemcpyDeviceToHost, ctx->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
    return e == cudaSuccess ? SPHNJ_OK : ck_cuda(ctx, e, "checkpoint save");
}

int sphnj_checkpoint_load(sphnj_ctx *ctx, const void *buffer, uint64_t bytes) {
    if (!ctx || !buffer) return SPHNJ_ERR_ARG;
    // a batch steps its scenes in lockstep: one scene's step cannot move alone
    if (ctx->batch) return ck_fail(ctx, SPHNJ_ERR_ARG, "the scene is in a batch: load before batching it");
    if (bytes < sizeof(CkHeader)) return ck_fail(ctx, SPHNJ_ERR_IO, "checkpoint shorter than its header");
    CkHeader h;
    std::memcpy(&h, buffer, sizeof h);
    if (std::memcmp(h.magic, kMagic, 8) != 0 || h.header_bytes != sizeof(CkHeader))
        return ck_fail(ctx, SPHNJ_ERR_IO, "not a checkpoint of this library version");
    // the arena layout depends on the counts, the grid and the form only; the
    // physical parameters are the loading context's own
    const sphnj_params &a = h.params, &b = ctx->p;
    if ((int)h.form != ctx->form || h.arena_bytes != ctx->arena_bytes ||
        a.fluid_number_total != b.fluid_number_total || a.solid_number != b.solid_number ||
        a.virt_number != b.virt_number || a.cell_number[0] != b.cell_number[0] ||
        a.cell_number[1] != b.cell_number[1] || a.cell_number_total != b.cell_number_total)
        return ck_fail(ctx, SPHNJ_ERR_ARG, "checkpoint of a context with other counts, grid or form");
    if (bytes < sizeof(CkHeader) + h.arena_bytes) return ck_fail(ctx, SPHNJ_ERR_IO, "checkpoint truncated");
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaStreamSynchronize(ctx->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->arena, static_cast<const char *>(buffer) + sizeof h, h.arena_bytes,
                            cudaMemcpyHostToDevice, ctx->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
    if (e != cudaSuccess) return ck_cuda(ctx, e, "checkpoint load");
    ctx->step = h.step;
    ctx->parity = h.parity;
    ctx->virt_sorted = h.virt_sorted != 0;
    ctx->virt_cells_valid = h.virt_cells_valid != 0;
    ctx->uploaded = true;
    ctx->d.rng_f = ctx->lf[ctx->parity].rng;  // current lists
    ctx->d.lst_f = ctx->lf[ctx->parity].lst;
    ctx->d.rng_s = ctx->ls[ctx->parity].rng;
    ctx->d.lst_s = ctx->ls[ctx->parity].lst;
    return SPHNJ_OK;
}

int sphnj_checkpoint_write(sphnj_ctx *ctx, const char *path) {
    if (!ctx || !path) return SPHNJ_ERR_ARG;
    uint64_t n = 0;
    sphnj_checkpoint_size(ctx, &n);
    std::vector<char> buf(n);
    int rc = sphnj_checkpoint_save(ctx, buf.data(), n);
    if (rc) return rc;
    FILE *f = std::fopen(path, "wb");
    if (!f) return ck_fail(ctx, SPHNJ_ERR_IO, "cannot open the checkpoint file for writing");
    const size_t w = std::fwrite(buf.data(), 1, n, f);
    const int closed = std::fclose(f);
    if (w != n || closed != 0) return ck_fail(ctx, SPHNJ_ERR_IO, "checkpoint file write failed");
    return SPHNJ_OK;
}

int sphnj_checkpoint_read(sphnj_ctx *ctx, const char *path) {
    if (!ctx || !path) return SPHNJ_ERR_ARG;
    FILE *f = std::fopen(path, "rb");
    if (!f) return ck_fail(ctx, SPHNJ_ERR_IO, "cannot open the checkpoint file");
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 0) {
        std::fclose(f);
        return ck_fail(ctx, SPHNJ_ERR_IO, "cannot size the checkpoint file");
    }
    std::vector<char> buf((size_t)n);
    const size_t r = std::fread(buf.data(), 1, (size_t)n, f);
    std::fclose(f);
    if (r != (size_t)n) return ck_fail(ctx, SPHNJ_ERR_IO, "checkpoint file read failed");
    return sphnj_checkpoint_load(ctx, buf.data(), (uint64_t)n);
}

}  // extern "C"
