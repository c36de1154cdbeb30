// C-ABI context of libsphnj: device arena, upload/download, and the step
// sequencer that issues the particle-step stages on one CUDA stream.
//
// Stage order per fluid step (DeviceCalculation::calculation,
// calculation.cu:28-43; outputs are the host driver's business):
//   1 cell ids                      particleCellUpdate    pair.cu:47-64
//   2 sort every sort_every_step    sortParticle          sort.cu:139-151
//     otherwise incremental lists   fillCell              pair.cu:170-181
//   3 solid coupling                coupleCalculation     solid.cu:494-507
//   4 virtual particles             virtUpdate            virt.cu:151-161
//   5 fluid pair pass + update      fluidCalculation      fluid.cu:289-302
//   6 k solid sub-steps             solidCalculation      solid.cu:473-492
//   7 S shifting passes             fluidCorrection       fluid.cu:442-459
// Nothing in a step reads device data on the host: the reference's per-step
// device-to-host copy of all fluid velocities (getMaxSpeed) is a device
// reduction here, and every launch is asynchronous on the context stream.
#include "context.h"

#include <algorithm>
#include <cstdio>
#include <cstring>

using namespace sphnj;

namespace {

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Two-pass arena carving: first pass sizes, second pass assigns.
struct Carver {
    char *base;
    size_t off = 0;
    template <class T> T *take(size_t n) {
        T *r = base ? reinterpret_cast<T *>(base + off) : nullptr;
        off += align256((n ? n : 1) * sizeof(T));
        return r;
    }
};

__global__ void k_u8_from_i32(uint8_t *dst, const int32_t *src, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (uint8_t)src[i];
}
__global__ void k_i32_from_u8(int32_t *dst, const uint8_t *src, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (int32_t)src[i];
}
__global__ void k_fill_u8(uint8_t *dst, uint8_t v, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = v;
}
__global__ void k_fill_dmat2(dmat2 *dst, dmat2 v, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = v;
}
__global__ void k_fill_f32(float *dst, float v, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = v;
}

}  // namespace

namespace sphnj {
void launch_u8_from_i32(cudaStream_t st, uint8_t *dst, const int32_t *src, int n) {
    if (n > 0) k_u8_from_i32<<<grid_for(n, 256), 256, 0, st>>>(dst, src, n);
}
void launch_i32_from_u8(cudaStream_t st, int32_t *dst, const uint8_t *src, int n) {
    if (n > 0) k_i32_from_u8<<<grid_for(n, 256), 256, 0, st>>>(dst, src, n);
}
void launch_fill_u8(cudaStream_t st, uint8_t *dst, uint8_t v, int n) {
    if (n > 0) k_fill_u8<<<grid_for(n, 256), 256, 0, st>>>(dst, v, n);
}
void launch_fill_dmat2(cudaStream_t st, dmat2 *dst, dmat2 v, int n) {
    if (n > 0) k_fill_dmat2<<<grid_for(n, 256), 256, 0, st>>>(dst, v, n);
}
void launch_fill_f32(cudaStream_t st, float *dst, float v, int n) {
    if (n > 0) k_fill_f32<<<grid_for(n, 256), 256, 0, st>>>(dst, v, n);
}
}  // namespace sphnj

namespace sphnj {

const char *const kStageNames[ST_COUNT] = {"bin", "sort", "rebuild", "capacity", "solid_couple", "virt_data",
                                           "fluid_pair", "fluid_update", "solid_deformation", "solid_force",
                                           "solid_update", "shift_pass", "shift_copy_back"};

cudaEvent_t Profiler::take() {
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void Profiler::enable(bool v) {
    for (auto &r : pending) {
        pool.push_back(r.a);
        pool.push_back(r.b);
    }
    pending.clear();
    on = v;
    for (int s = 0; s < ST_COUNT; ++s) ms[s] = 0.0, calls[s] = kernels[s] = 0;
}

cudaError_t Profiler::collect() {
    for (auto &r : pending) {
        float t = 0.0f;
        cudaError_t e = cudaEventElapsedTime(&t, r.a, r.b);
        if (e != cudaSuccess) return e;
        ms[r.stage] += t;
        calls[r.stage] += 1;
        kernels[r.stage] += r.kernels;
        pool.push_back(r.a);
        pool.push_back(r.b);
    }
    pending.clear();
    return cudaSuccess;
}

void Profiler::release() {
    for (auto &r : pending) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    pending.clear();
    for (auto e : pool) cudaEventDestroy(e);
    pool.clear();
}

}  // namespace sphnj

namespace {

int fail(sphnj_ctx *c, int code, const std::string &m) {
    if (c) c->msg = m;
    return code;
}

int cuda_fail(sphnj_ctx *c, cudaError_t e, const char *where) {
    return fail(c, SPHNJ_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                       \
    do {                                                               \
        cudaError_t e_ = (call);                                       \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);       \
    } while (0)

size_t layout(sphnj_ctx *ctx, char *base) {
    const sphnj_params &p = ctx->p;
    const int nf = p.fluid_number_total, ns = p.solid_number, nv = p.virt_number, C = p.cell_number_total;
    const int nmax = std::max(nf, std::max(ns, nv));
    Carver a{base};
    DevState &d = ctx->d;
    d.f_pos = a.take<float2>(nf); d.f_vel = a.take<float2>(nf);
    d.f_grad = a.take<float2>(nf); d.f_dudt = a.take<float2>(nf);
    d.f_rho = a.take<float>(nf); d.f_p = a.take<float>(nf);
    d.f_color = a.take<float>(nf); d.f_drho = a.take<float>(nf);
    d.f_dudx = a.take<float4>(nf);
    d.f_phase = a.take<uint8_t>(nf); d.f_fbt = a.take<uint8_t>(nf); d.f_near = a.take<uint8_t>(nf);
    d.f_cell = a.take<int>(nf);
    d.f_x_alt = a.take<float2>(nf);
    d.f_xl = a.take<float2>(nf);
    d.f_xl_alt = a.take<float2>(nf);
    d.f_celll = a.take<int>(nf);
    d.f_btl = a.take<uint8_t>(nf);
    d.f_listed = a.take<int>(nf);
    ctx->f_listed_total = a.take<int>(1);
    d.f_listed_total = ctx->f_listed_total;
    d.f_nbr = a.take<uint4>((size_t)kNbrChunks * nf);
    d.f_nbr_cnt = a.take<uint8_t>(nf);
    d.disp2_bits = a.take<unsigned int>(1 + kMaskShifts);
    d.stamp = a.take<int>(1);
    d.s_pos = a.take<double2>(ns); d.s_ref = a.take<double2>(ns);
    d.s_vel = a.take<double2>(ns); d.s_dudt = a.take<double2>(ns);
    d.s_F = a.take<dmat2>(ns); d.s_P = a.take<dmat2>(ns); d.s_L = a.take<dmat2>(ns);
    d.s_maxstrain = a.take<dmat2>(ns);
    d.s_p = a.take<float>(ns); d.s_normal = a.take<float2>(ns); d.s_couple = a.take<float2>(ns);
    d.s_bt = a.take<uint8_t>(ns); d.s_mat = a.take<uint8_t>(ns); d.s_cell = a.take<int>(ns);
    d.v_pos = a.take<float2>(nv); d.v_normal = a.take<float2>(nv); d.v_vel = a.take<float2>(nv);
    d.v_p = a.take<float>(nv); d.v_rho = a.take<float>(nv);
    d.v_phase = a.take<uint8_t>(nv); d.v_bt = a.take<uint8_t>(nv); d.v_cell = a.take<int>(nv);
    for (int k = 0; k < 2; ++k) {
        ctx->lf[k].rng = a.take<int2>(C); ctx->lf[k].lst = a.take<int>(nf);
        ctx->ls[k].rng = a.take<int2>(C); ctx->ls[k].lst = a.take<int>(ns);
    }
    ctx->lv.rng = a.take<int2>(C); ctx->lv.lst = a.take<int>(nv);
    const bool mixed = ctx->form == SPHNJ_FORM_MIXED;
    if (mixed) {
        d.f_off = a.take<float2>(nf); d.f_offc = a.take<float2>(nf); d.f_velc = a.take<float2>(nf);
        d.f_x0l = a.take<float2>(nf); d.f_xc0l = a.take<float2>(nf); d.f_offcl = a.take<float2>(nf);
        d.s_rc = a.take<int2>(ns);
        d.s_roff = a.take<float2>(ns); d.s_u = a.take<float2>(ns); d.s_uc = a.take<float2>(ns);
        d.s_v = a.take<float2>(ns); d.s_vc = a.take<float2>(ns); d.s_off = a.take<float2>(ns);
        d.s_acc = a.take<float2>(ns);
        d.s_PL = a.take<float4>(ns); d.s_FL = a.take<float4>(ns);
        d.s_nbr = a.take<int>((size_t)kSolidNbrCap * ns); d.s_nbr_cnt = a.take<uint8_t>(ns);
        d.v_off = a.take<float2>(nv);
    }
    ctx->sc.cnt9 = a.take<int>((size_t)9 * C);
    ctx->sc.cnt = a.take<int>(C);
    ctx->sc.local = a.take<int>(C);
    ctx->sc.sums = a.take<int>(SCAN_MAX_TILES);
    ctx->sc.cursor = a.take<int>(C);
    ctx->sc.bucket = a.take<int>(nmax);
    ctx->sc.sorted = a.take<int>(nmax);
    // sort payload staging: the per-kind column sets of kernels_cells.cu
    const size_t pf = mixed ? 54 : 30, ps = mixed ? 142 : 86, pv = mixed ? 29 : 21;
    size_t pay = std::max((size_t)nf * pf, std::max((size_t)ns * ps, (size_t)nv * pv)) + 16 * 256;
    ctx->payload = a.take<char>(pay);
    d.tile_list = a.take<int>(C);  // at most one tile per cell (tile height >= 1)
    d.tile_count = a.take<int>(1);
    d.max_speed2_bits = a.take<unsigned int>(1);
    d.err = a.take<DevErr>(1);
    ctx->diag_part = a.take<double>((size_t)kDiagBlocks * kDiagSlots);
    ctx->diag_out = a.take<sphnj_diag>(1);
    return a.off;
}

void bind_lists(const sphnj_ctx *ctx, DevState &d, int parity) {
    d.rng_f = ctx->lf[parity].rng;
    d.lst_f = ctx->lf[parity].lst;
    d.rng_s = ctx->ls[parity].rng;
    d.lst_s = ctx->ls[parity].lst;
    d.rng_v = ctx->lv.rng;
    d.lst_v = ctx->lv.lst;
}
void bind_lists(sphnj_ctx *ctx) { bind_lists(ctx, ctx->d, ctx->parity); }

}  // namespace

namespace sphnj {

Scene scene_of(const sphnj_ctx *ctx, int parity) {
    Scene s{};
    s.p = ctx->p;
    s.d = ctx->d;
    bind_lists(ctx, s.d, parity);
    for (int k = 0; k < 2; ++k) {
        s.lf[k] = ctx->lf[k];
        s.ls[k] = ctx->ls[k];
    }
    s.lv = ctx->lv;
    s.sc = ctx->sc;
    s.payload = static_cast<char *>(ctx->payload);
    s.f_listed_total = ctx->f_listed_total;
    s.tile_h = ctx->tiles.tile_h;
    s.lists = ctx->tiles.lists ? 1 : 0;
    return s;
}

int check_device_error(sphnj_ctx *ctx) {
    CK(cudaMemcpyAsync(ctx->h_err, ctx->d.err, sizeof(DevErr), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return device_error_status(ctx);
}

int device_error_status(sphnj_ctx *ctx) {
    const DevErr &e = *ctx->h_err;
    if (e.code == 0) return SPHNJ_OK;
    char buf[256];
    switch (e.code) {
    case SPHNJ_ERR_OUT_OF_GRID:
        snprintf(buf, sizeof buf, "particle outside the cell grid (kind %d, index %d, cell id %d)", e.info[0],
                 e.info[1], e.info[2]);
        break;
    case SPHNJ_ERR_NONFINITE:
        snprintf(buf, sizeof buf, "non-finite state (kind %d, index %d) after an update", e.info[0], e.info[1]);
        break;
    case SPHNJ_ERR_CELL_OVERFLOW:
        snprintf(buf, sizeof buf, "cell %d holds %d particles, more than the reference's %d slots", e.info[0],
                 e.info[1], SPHNJ_CELL_SIZE);
        break;
    default:
        snprintf(buf, sizeof buf, "device error %d (%d %d %d)", e.code, e.info[0], e.info[1], e.info[2]);
    }
    return fail(ctx, e.code, buf);
}

}  // namespace sphnj

namespace {

template <class T> int h2d(sphnj_ctx *ctx, T *dst, const void *src, size_t n) {
    if (n == 0) return SPHNJ_OK;
    CK(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, ctx->st));
    return SPHNJ_OK;
}
template <class T> int d2h(sphnj_ctx *ctx, void *dst, const T *src, size_t n) {
    if (n == 0 || !dst) return SPHNJ_OK;
    CK(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->st));
    return SPHNJ_OK;
}
// 32-bit enum array on the host <-> uint8 on the device, through the bucket
// scratch (free outside a step).
int enum_h2d(sphnj_ctx *ctx, uint8_t *dst, const int32_t *src, int n) {
    if (n == 0) return SPHNJ_OK;
    CK(cudaMemcpyAsync(ctx->sc.bucket, src, n * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->st));
    launch_u8_from_i32(ctx->st, dst, ctx->sc.bucket, n);
    // the staging buffer is reused by the next field: order through the stream
    return SPHNJ_OK;
}
int enum_d2h(sphnj_ctx *ctx, int32_t *dst, const uint8_t *src, int n) {
    if (n == 0 || !dst) return SPHNJ_OK;
    launch_i32_from_u8(ctx->st, ctx->sc.bucket, src, n);
    CK(cudaMemcpyAsync(dst, ctx->sc.bucket, n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));  // staging reused by the next field
    return SPHNJ_OK;
}

#define RET(x)                      \
    do {                            \
        int r_ = (x);               \
        if (r_) return r_;          \
    } while (0)

// The fluid kinematics (mask bit) and densities / pressures (thermo bit) of s
// that lie in sphnj_host_alloc memory, aligned for the kernel's float2 /
// float accesses.
bool kernel_access(const void *ptr, size_t bytes, size_t align) {
    return ptr && reinterpret_cast<uintptr_t>(ptr) % align == 0 && host_mapped(ptr, bytes);
}
FluidHost fluid_host(uint32_t mask, const sphnj_host_state *s, int nf) {
    FluidHost h{};
    if (nf <= 0) return h;
    const size_t n = (size_t)nf;
    if (mask & SPHNJ_F_FLUID_KINEMATICS) {
        if (kernel_access(s->fluid_position, n * sizeof(float2), alignof(float2)))
            h.pos = reinterpret_cast<float2 *>(s->fluid_position);
        if (kernel_access(s->fluid_velocity, n * sizeof(float2), alignof(float2)))
            h.vel = reinterpret_cast<float2 *>(s->fluid_velocity);
    }
    if (mask & SPHNJ_F_FLUID_THERMO) {
        if (kernel_access(s->fluid_density, n * sizeof(float), alignof(float))) h.rho = s->fluid_density;
        if (kernel_access(s->fluid_pressure, n * sizeof(float), alignof(float))) h.p = s->fluid_pressure;
    }
    return h;
}

}  // namespace

extern "C" {

int sphnj_create(const sphnj_params *p, int form, sphnj_ctx **out) {
    if (!p || !out) return SPHNJ_ERR_ARG;
    *out = nullptr;
    if (form != SPHNJ_FORM_PLAIN && form != SPHNJ_FORM_MIXED) return SPHNJ_ERR_UNSUPPORTED;
    if (p->fluid_number_total < 0 || p->solid_number < 0 || p->virt_number < 0) return SPHNJ_ERR_ARG;
    if (p->cell_number[0] < 3 || p->cell_number[1] < 3 ||
        (long)p->cell_number[0] * p->cell_number[1] != p->cell_number_total)
        return SPHNJ_ERR_ARG;
    if ((p->cell_number_total + SCAN_TILE - 1) / SCAN_TILE > SCAN_MAX_TILES) return SPHNJ_ERR_UNSUPPORTED;
    if (p->sort_every_step < 1 || p->solid_sub_step < 1 || p->shift_per_step < 0) return SPHNJ_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return SPHNJ_ERR_NO_DEVICE;
    }
    sphnj_ctx *ctx = new sphnj_ctx;
    ctx->p = *p;
    ctx->form = form;
    cudaGetDevice(&ctx->device);
    ctx->arena_bytes = layout(ctx, nullptr);
    cudaError_t e = cudaMalloc(&ctx->arena, ctx->arena_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return SPHNJ_ERR_CUDA;
    }
    layout(ctx, ctx->arena);
    if (cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost(&ctx->h_err, sizeof(DevErr)) != cudaSuccess) {
        cudaGetLastError();
        sphnj_destroy(ctx);
        return SPHNJ_ERR_CUDA;
    }
    ctx->st = ctx->own;
    if (cudaMemsetAsync(ctx->arena, 0, ctx->arena_bytes, ctx->st) != cudaSuccess ||
        cudaStreamSynchronize(ctx->st) != cudaSuccess) {
        sphnj_destroy(ctx);
        return SPHNJ_ERR_CUDA;
    }
    if (configure_sweeps(ctx->tiles) != cudaSuccess) {
        sphnj_destroy(ctx);
        return SPHNJ_ERR_CUDA;
    }
    bind_lists(ctx);
    *out = ctx;
    return SPHNJ_OK;
}

void sphnj_destroy(sphnj_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    ctx->prof.release();
    if (ctx->probe_buf) cudaFree(ctx->probe_buf);
    for (auto &g : ctx->graphs) cudaGraphExecDestroy(g.second.exec);
    if (ctx->arena) cudaFree(ctx->arena);
    if (ctx->h_err) cudaFreeHost(ctx->h_err);
    if (ctx->io_st) {
        cudaStreamSynchronize(ctx->io_st);
        cudaStreamDestroy(ctx->io_st);
    }
    for (cudaEvent_t e : {ctx->ev_start, ctx->ev_in, ctx->ev_rho_p, ctx->ev_out})
        if (e) cudaEventDestroy(e);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    delete ctx;
}

int sphnj_set_stream(sphnj_ctx *ctx, void *stream) {
    if (!ctx) return SPHNJ_ERR_ARG;
    if (ctx->batch) return fail(ctx, SPHNJ_ERR_ARG, "the scene is in a batch: set the batch's stream");
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->st));
    ctx->st = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    return SPHNJ_OK;
}

int sphnj_upload(sphnj_ctx *ctx, const sphnj_host_state *s) {
    if (!ctx || !s) return SPHNJ_ERR_ARG;
    cudaSetDevice(ctx->device);
    const sphnj_params &p = ctx->p;
    const int nf = p.fluid_number_total, ns = p.solid_number, nv = p.virt_number, C = p.cell_number_total;
    DevState &d = ctx->d;
    cudaStream_t st = ctx->st;
    // fluid (host_data.cuh:24-46)
    if (s->fluid_position) RET(h2d(ctx, d.f_pos, s->fluid_position, nf)); else CK(cudaMemsetAsync(d.f_pos, 0, 8ul * nf, st));
    if (s->fluid_velocity) RET(h2d(ctx, d.f_vel, s->fluid_velocity, nf)); else CK(cudaMemsetAsync(d.f_vel, 0, 8ul * nf, st));
    if (s->fluid_density) RET(h2d(ctx, d.f_rho, s->fluid_density, nf)); else CK(cudaMemsetAsync(d.f_rho, 0, 4ul * nf, st));
    if (s->fluid_pressure) RET(h2d(ctx, d.f_p, s->fluid_pressure, nf)); else CK(cudaMemsetAsync(d.f_p, 0, 4ul * nf, st));
    if (s->fluid_phase) RET(enum_h2d(ctx, d.f_phase, s->fluid_phase, nf)); else CK(cudaMemsetAsync(d.f_phase, 0, nf, st));
    if (s->fluid_boundary_type) RET(enum_h2d(ctx, d.f_fbt, s->fluid_boundary_type, nf));
    else launch_fill_u8(st, d.f_fbt, SPHNJ_FREE_SURFACE, nf);
    if (s->fluid_has_near_particle) RET(enum_h2d(ctx, d.f_near, s->fluid_has_near_particle, nf));
    else CK(cudaMemsetAsync(d.f_near, SPHNJ_NO_PARTICLE, nf, st));
    if (s->fluid_du_dx) RET(h2d(ctx, d.f_dudx, s->fluid_du_dx, nf)); else CK(cudaMemsetAsync(d.f_dudx, 0, 16ul * nf, st));
    if (s->fluid_gradient) RET(h2d(ctx, d.f_grad, s->fluid_gradient, nf)); else CK(cudaMemsetAsync(d.f_grad, 0, 8ul * nf, st));
    if (s->fluid_du_dt) RET(h2d(ctx, d.f_dudt, s->fluid_du_dt, nf)); else CK(cudaMemsetAsync(d.f_dudt, 0, 8ul * nf, st));
    if (s->fluid_color) RET(h2d(ctx, d.f_color, s->fluid_color, nf)); else CK(cudaMemsetAsync(d.f_color, 0, 4ul * nf, st));
    if (s->fluid_drho_dt) RET(h2d(ctx, d.f_drho, s->fluid_drho_dt, nf)); else CK(cudaMemsetAsync(d.f_drho, 0, 4ul * nf, st));
    // solid (host_data.cuh:64-87)
    const dmat2 I = {1.0, 0.0, 0.0, 1.0}, Z = {0.0, 0.0, 0.0, 0.0};
    const dmat2 MS = {-(double)p.yield_strain, 0.0, 0.0, -(double)p.yield_strain};
    if (s->solid_position) RET(h2d(ctx, d.s_pos, s->solid_position, ns)); else CK(cudaMemsetAsync(d.s_pos, 0, 16ul * ns, st));
    if (s->solid_reference_position) RET(h2d(ctx, d.s_ref, s->solid_reference_position, ns));
    else CK(cudaMemsetAsync(d.s_ref, 0, 16ul * ns, st));
    if (s->solid_velocity) RET(h2d(ctx, d.s_vel, s->solid_velocity, ns)); else CK(cudaMemsetAsync(d.s_vel, 0, 16ul * ns, st));
    if (s->solid_boundary_type) RET(enum_h2d(ctx, d.s_bt, s->solid_boundary_type, ns)); else CK(cudaMemsetAsync(d.s_bt, 0, ns, st));
    if (s->solid_material_type) RET(enum_h2d(ctx, d.s_mat, s->solid_material_type, ns)); else CK(cudaMemsetAsync(d.s_mat, 0, ns, st));
    if (s->solid_max_strain) RET(h2d(ctx, d.s_maxstrain, s->solid_max_strain, ns)); else launch_fill_dmat2(st, d.s_maxstrain, MS, ns);
    if (s->solid_pressure) RET(h2d(ctx, d.s_p, s->solid_pressure, ns)); else CK(cudaMemsetAsync(d.s_p, 0, 4ul * ns, st));
    if (s->solid_deformation) RET(h2d(ctx, d.s_F, s->solid_deformation, ns)); else launch_fill_dmat2(st, d.s_F, I, ns);
    if (s->solid_stress_1st_piola) RET(h2d(ctx, d.s_P, s->solid_stress_1st_piola, ns)); else launch_fill_dmat2(st, d.s_P, Z, ns);
    if (s->solid_correction) RET(h2d(ctx, d.s_L, s->solid_correction, ns)); else launch_fill_dmat2(st, d.s_L, I, ns);
    if (s->solid_du_dt) RET(h2d(ctx, d.s_dudt, s->solid_du_dt, ns)); else CK(cudaMemsetAsync(d.s_dudt, 0, 16ul * ns, st));
    if (s->solid_normal) RET(h2d(ctx, d.s_normal, s->solid_normal, ns)); else CK(cudaMemsetAsync(d.s_normal, 0, 8ul * ns, st));
    if (s->solid_couple_dudt) RET(h2d(ctx, d.s_couple, s->solid_couple_dudt, ns)); else CK(cudaMemsetAsync(d.s_couple, 0, 8ul * ns, st));
    // virtual (host_data.cuh:99-115)
    if (s->virt_position) RET(h2d(ctx, d.v_pos, s->virt_position, nv)); else CK(cudaMemsetAsync(d.v_pos, 0, 8ul * nv, st));
    if (s->virt_velocity) RET(h2d(ctx, d.v_vel, s->virt_velocity, nv)); else CK(cudaMemsetAsync(d.v_vel, 0, 8ul * nv, st));
    if (s->virt_pressure) RET(h2d(ctx, d.v_p, s->virt_pressure, nv)); else CK(cudaMemsetAsync(d.v_p, 0, 4ul * nv, st));
    if (s->virt_density) RET(h2d(ctx, d.v_rho, s->virt_density, nv)); else launch_fill_f32(st, d.v_rho, p.reference_density[0], nv);
    if (s->virt_phase) RET(enum_h2d(ctx, d.v_phase, s->virt_phase, nv)); else CK(cudaMemsetAsync(d.v_phase, SPHNJ_LIQUID, nv, st));
    if (s->virt_boundary_type) RET(enum_h2d(ctx, d.v_bt, s->virt_boundary_type, nv)); else CK(cudaMemsetAsync(d.v_bt, 0, nv, st));
    // cell lists start empty (Cell(), cell.cuh:31-46)
    for (int k = 0; k < 2; ++k) {
        CK(cudaMemsetAsync(ctx->lf[k].rng, 0, sizeof(int2) * C, st));
        CK(cudaMemsetAsync(ctx->ls[k].rng, 0, sizeof(int2) * C, st));
    }
    CK(cudaMemsetAsync(ctx->lv.rng, 0, sizeof(int2) * C, st));
    CK(cudaMemsetAsync(d.f_listed, 0xFF, sizeof(int) * (size_t)nf, st));
    CK(cudaMemsetAsync(ctx->f_listed_total, 0, sizeof(int), st));
    CK(cudaMemsetAsync(d.err, 0, sizeof(DevErr), st));
    CK(cudaMemsetAsync(d.max_speed2_bits, 0, sizeof(unsigned), st));
    ctx->parity = 0;
    ctx->virt_sorted = false;
    ctx->virt_cells_valid = false;
    ctx->step = p.istart;
    bind_lists(ctx);
    // wall normals once before the loop (virtNormalCalculation, calculation.cu:28)
    GroupOne g{scene_of(ctx, ctx->parity), ctx->form};
    if (s->virt_normal) {
        RET(h2d(ctx, d.v_normal, s->virt_normal, nv));
    } else if (nv > 0) {
        launch_virt_normal(st, g);
        // the virtual lists it built go: the step starts from empty lists
        CK(cudaMemsetAsync(ctx->lv.rng, 0, sizeof(int2) * C, st));
    }
    // mixed form: cells + offsets, displacements and compensations
    if (ctx->form == SPHNJ_FORM_MIXED) launch_mixed_split(st, g, 7);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    ctx->uploaded = true;
    return SPHNJ_OK;
}

}  // extern "C"

namespace sphnj {

template <class G>
int issue_step(G &g, const StepKind &k, cudaStream_t st, const TileConfig &tc, Profiler *prof, const StepIO *io) {
    int launched = 0;
    // Under stream capture the event operations become external event nodes,
    // so that one graph serves every call; direct launches use them as they are.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (io && k.io) cudaStreamIsCapturing(st, &cap);
    const bool capturing = cap == cudaStreamCaptureStatusActive;
    auto wait_inputs = [&] {
        if (io && io->in && (k.io & 1))
            cudaStreamWaitEvent(st, io->in, capturing ? cudaEventWaitExternal : cudaEventWaitDefault);
    };
    auto stage = [&](int s, auto &&fn) {
        Profiler::Rec r{s, 0, nullptr, nullptr};
        if (prof) {
            r.a = prof->take();
            r.b = prof->take();
            cudaEventRecord(r.a, st);
        }
        r.kernels = fn();
        if (prof) {
            cudaEventRecord(r.b, st);
            prof->pending.push_back(r);
        }
        launched += r.kernels;
    };
    auto fluid = [](const sphnj_params &p) { return p.fluid_number_total > 0; };
    auto solid = [](const sphnj_params &p) { return p.solid_number > 0; };
    auto virt = [](const sphnj_params &p) { return p.virt_number > 0; };
    const bool any_fluid = g.any(fluid), any_solid = g.any(solid);
    stage(ST_BIN, [&] { return launch_bin(st, g, k.bin_virt); });
    if (k.is_sort) {
        wait_inputs();  // the sort moves every fluid field
        if (any_fluid) stage(ST_SORT, [&] { return launch_sort_kind(st, g, KF, k.parity); });
        if (any_solid) stage(ST_SORT, [&] { return launch_sort_kind(st, g, KS, k.parity); });
        if (k.sort_virt) stage(ST_SORT, [&] { return launch_sort_kind(st, g, KV, k.parity); });
    } else {
        if (any_fluid) stage(ST_REBUILD, [&] { return launch_rebuild_kind(st, g, KF, k.parity); });
        if (any_solid) stage(ST_REBUILD, [&] { return launch_rebuild_kind(st, g, KS, k.parity); });
    }
    stage(ST_CAPACITY, [&] { return launch_capacity_check(st, g); });
    if (!k.is_sort) wait_inputs();  // binning and the list rebuild read positions only
    if (g.any([](const sphnj_params &p) { return p.fluid_number_total > 0 && p.solid_number > 0; }))
        stage(ST_SOLID_COUPLE, [&] { return launch_solid_couple(st, g); });
    if (g.any(virt)) stage(ST_VIRT_DATA, [&] { return launch_virt_data(st, g); });
    if (any_fluid) {
        stage(ST_FLUID_PAIR, [&] { return launch_fluid_pair(st, g, tc); });
        stage(ST_FLUID_UPDATE, [&] { return launch_fluid_update(st, g); });
    }
    if (io && io->rho_p && (k.io & 2))
        cudaEventRecordWithFlags(io->rho_p, st, capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
    int subs = 0, shifts = 0;
    g.any([&](const sphnj_params &p) {
        if (p.solid_number > 0) subs = std::max(subs, p.solid_sub_step);
        if (p.fluid_number_total > 0) shifts = std::max(shifts, p.shift_per_step);
        return false;
    });
    for (int s = 0; s < subs; ++s) {
        stage(ST_SOLID_DEFORM, [&] { return launch_solid_deformation(st, g, s); });
        stage(ST_SOLID_FORCE, [&] { return launch_solid_force(st, g, s); });
        stage(ST_SOLID_UPDATE, [&] { return launch_solid_update(st, g, s); });
    }
    for (int s = 0; s < shifts; ++s) stage(ST_SHIFT_PASS, [&] { return launch_shift_pass(st, g, tc, s); });
    if (shifts) stage(ST_SHIFT_COPY_BACK, [&] { return launch_shift_copy_back(st, g); });
    return launched;
}

template int issue_step<GroupOne>(GroupOne &, const StepKind &, cudaStream_t, const TileConfig &, Profiler *,
                                  const StepIO *);
template int issue_step<GroupMany>(GroupMany &, const StepKind &, cudaStream_t, const TileConfig &, Profiler *,
                                   const StepIO *);

StepKind next_kind(const sphnj_ctx *ctx) {
    const sphnj_params &p = ctx->p;
    const int step = ctx->step + 1;
    StepKind k;
    k.is_sort = ((step - 1) % p.sort_every_step) == 0;  // SimTime::isSort
    // virtual particles are binned until their first sort (and once after an
    // upload); afterwards their ids never change.  After their first sort
    // their order and lists stay as they are (a stable sort of sorted keys is
    // the identity), so they are sorted once.
    k.bin_virt = !ctx->virt_sorted || !ctx->virt_cells_valid;
    k.sort_virt = k.is_sort && p.virt_number > 0 && !ctx->virt_sorted;
    k.parity = k.is_sort ? ctx->parity : ctx->parity ^ 1;
    return k;
}

void commit_step(sphnj_ctx *ctx, const StepKind &k) {
    ctx->step++;
    ctx->parity = k.parity;
    ctx->virt_cells_valid = true;
    if (k.sort_virt) ctx->virt_sorted = true;
    bind_lists(ctx);
}

}  // namespace sphnj

namespace {

void drop_graphs(sphnj_ctx *ctx) {
    for (auto &g : ctx->graphs) cudaGraphExecDestroy(g.second.exec);
    ctx->graphs.clear();
}

}  // namespace

namespace {

// Issues n steps of ctx on its stream (a captured graph per kind of step,
// unless graphs are off or the stages are being timed); io_first / io_last
// are the StepKind::io bits of the first and the last step.
int run_steps(sphnj_ctx *ctx, int n, int io_first = 0, int io_last = 0) {
    cudaStream_t st = ctx->st;
    const StepIO io{ctx->ev_in, ctx->ev_rho_p};
    for (int it = 0; it < n; ++it) {
        StepKind k = next_kind(ctx);
        k.io = (it == 0 ? io_first : 0) | (it == n - 1 ? io_last : 0);
        GroupOne g{scene_of(ctx, k.parity), ctx->form};
        g.pdl = ctx->pdl;
        if (ctx->use_graphs && !ctx->prof.on) {
            auto it_g = ctx->graphs.find(k.key());
            if (it_g == ctx->graphs.end()) {
                cudaGraph_t graph = nullptr;
                CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                const int launched = issue_step(g, k, st, ctx->tiles, nullptr, &io);
                cudaError_t e = cudaStreamEndCapture(st, &graph);
                cudaGraphExec_t exec = nullptr;
                if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
                if (graph) cudaGraphDestroy(graph);
                if (e != cudaSuccess) return cuda_fail(ctx, e, "step graph capture");
                it_g = ctx->graphs.emplace(k.key(), StepGraph{exec, launched}).first;
            }
            CK(cudaGraphLaunch(it_g->second.exec, st));
            ctx->launches += (uint64_t)it_g->second.kernels;
        } else {
            ctx->launches += (uint64_t)issue_step(g, k, st, ctx->tiles, ctx->prof.on ? &ctx->prof : nullptr, &io);
        }
        CK(cudaGetLastError());
        commit_step(ctx, k);
    }
    return SPHNJ_OK;
}

}  // namespace

extern "C" int sphnj_step(sphnj_ctx *ctx, int n) {
    if (!ctx || n < 0) return SPHNJ_ERR_ARG;
    if (!ctx->uploaded) return fail(ctx, SPHNJ_ERR_ARG, "sphnj_step before sphnj_upload");
    if (ctx->batch) return fail(ctx, SPHNJ_ERR_ARG, "the scene is in a batch: step the batch");
    cudaSetDevice(ctx->device);
    return run_steps(ctx, n);
}

extern "C" {

int sphnj_set_launch_chaining(sphnj_ctx *ctx, int on) {
    if (!ctx) return SPHNJ_ERR_ARG;
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->st));
    ctx->pdl = on != 0;
    drop_graphs(ctx);
    return SPHNJ_OK;
}

int sphnj_set_graphs(sphnj_ctx *ctx, int on) {
    if (!ctx) return SPHNJ_ERR_ARG;
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->st));
    ctx->use_graphs = on != 0;
    drop_graphs(ctx);
    return SPHNJ_OK;
}

}  // extern "C"

namespace {

// Fields of sphnj_step_exchange's transfers that move on its second stream.
enum Deferred : uint32_t { DEF_VEL = 1u, DEF_RHO = 2u, DEF_P = 4u };

// sphnj_upload_fields without the final synchronisation; the fluid fields
// in `defer` are left out (the caller moves them).
int upload_fields_enqueue(sphnj_ctx *ctx, uint32_t mask, const sphnj_host_state *s, uint32_t defer) {
    const sphnj_params &p = ctx->p;
    const int nf = p.fluid_number_total, ns = p.solid_number, nv = p.virt_number;
    DevState &d = ctx->d;
    // Mixed form: the host-layout mirrors are refreshed from the state first,
    // so that a kind whose positions are re-split keeps its other fields; only
    // kinds whose positions are given are re-split (a round trip through an
    // absolute FP32 position would lose the offset's precision).
    const bool mixed = ctx->form == SPHNJ_FORM_MIXED;
    // fluid fields in device-mapped host memory: one kernel, no copies
    FluidHost fh = fluid_host(mask, s, nf);
    if (defer & DEF_VEL) fh.vel = nullptr;
    if (defer & DEF_RHO) fh.rho = nullptr;
    if (defer & DEF_P) fh.p = nullptr;
    int resplit = 0;
    if (mixed) {
        if ((mask & SPHNJ_F_FLUID_KINEMATICS) && s->fluid_position && !fh.pos) resplit |= 1;
        if ((mask & SPHNJ_F_SOLID_KINEMATICS) &&
            (s->solid_position || s->solid_reference_position || s->solid_velocity))
            resplit |= 2;
        // (a re-split fluid reads only the positions it is given)
        launch_mixed_join(ctx->st, GroupOne{scene_of(ctx, ctx->parity), ctx->form}, resplit & 2);
        if ((mask & SPHNJ_F_FLUID_KINEMATICS) && s->fluid_velocity && !s->fluid_position && !fh.vel)
            CK(cudaMemsetAsync(d.f_velc, 0, sizeof(float2) * (size_t)nf, ctx->st));
    }
    launch_fluid_from_host(ctx->st, GroupOne{scene_of(ctx, ctx->parity), ctx->form}, fh);
    if (mask & SPHNJ_F_FLUID_KINEMATICS) {
        if (s->fluid_position && !fh.pos) RET(h2d(ctx, d.f_pos, s->fluid_position, nf));
        if (s->fluid_velocity && !fh.vel && !(defer & DEF_VEL)) RET(h2d(ctx, d.f_vel, s->fluid_velocity, nf));
    }
    if (mask & SPHNJ_F_FLUID_THERMO) {
        if (s->fluid_density && !fh.rho && !(defer & DEF_RHO)) RET(h2d(ctx, d.f_rho, s->fluid_density, nf));
        if (s->fluid_pressure && !fh.p && !(defer & DEF_P)) RET(h2d(ctx, d.f_p, s->fluid_pressure, nf));
        if (s->fluid_phase) RET(enum_h2d(ctx, d.f_phase, s->fluid_phase, nf));
    }
    if (mask & SPHNJ_F_FLUID_FLAGS) {
        if (s->fluid_boundary_type) RET(enum_h2d(ctx, d.f_fbt, s->fluid_boundary_type, nf));
        if (s->fluid_has_near_particle) RET(enum_h2d(ctx, d.f_near, s->fluid_has_near_particle, nf));
    }
    if (mask & SPHNJ_F_FLUID_DERIVED) {
        if (s->fluid_du_dx) RET(h2d(ctx, d.f_dudx, s->fluid_du_dx, nf));
        if (s->fluid_gradient) RET(h2d(ctx, d.f_grad, s->fluid_gradient, nf));
        if (s->fluid_du_dt) RET(h2d(ctx, d.f_dudt, s->fluid_du_dt, nf));
        if (s->fluid_color) RET(h2d(ctx, d.f_color, s->fluid_color, nf));
        if (s->fluid_drho_dt) RET(h2d(ctx, d.f_drho, s->fluid_drho_dt, nf));
    }
    if (mask & SPHNJ_F_SOLID_KINEMATICS) {
        if (s->solid_position) RET(h2d(ctx, d.s_pos, s->solid_position, ns));
        if (s->solid_reference_position) RET(h2d(ctx, d.s_ref, s->solid_reference_position, ns));
        if (s->solid_velocity) RET(h2d(ctx, d.s_vel, s->solid_velocity, ns));
    }
    if (mask & SPHNJ_F_SOLID_MATERIAL) {
        if (s->solid_boundary_type) RET(enum_h2d(ctx, d.s_bt, s->solid_boundary_type, ns));
        if (s->solid_material_type) RET(enum_h2d(ctx, d.s_mat, s->solid_material_type, ns));
        if (s->solid_max_strain) RET(h2d(ctx, d.s_maxstrain, s->solid_max_strain, ns));
    }
    if (mask & SPHNJ_F_SOLID_DERIVED) {
        if (s->solid_pressure) RET(h2d(ctx, d.s_p, s->solid_pressure, ns));
        if (s->solid_deformation) RET(h2d(ctx, d.s_F, s->solid_deformation, ns));
        if (s->solid_stress_1st_piola) RET(h2d(ctx, d.s_P, s->solid_stress_1st_piola, ns));
        if (s->solid_correction) RET(h2d(ctx, d.s_L, s->solid_correction, ns));
        if (s->solid_du_dt) RET(h2d(ctx, d.s_dudt, s->solid_du_dt, ns));
        if (s->solid_normal) RET(h2d(ctx, d.s_normal, s->solid_normal, ns));
        if (s->solid_couple_dudt) RET(h2d(ctx, d.s_couple, s->solid_couple_dudt, ns));
    }
    if (mask & SPHNJ_F_VIRT) {
        // positions of virtual particles are fixed after their first sort
        if (s->virt_normal) RET(h2d(ctx, d.v_normal, s->virt_normal, nv));
        if (s->virt_velocity) RET(h2d(ctx, d.v_vel, s->virt_velocity, nv));
        if (s->virt_pressure) RET(h2d(ctx, d.v_p, s->virt_pressure, nv));
        if (s->virt_density) RET(h2d(ctx, d.v_rho, s->virt_density, nv));
        if (s->virt_phase) RET(enum_h2d(ctx, d.v_phase, s->virt_phase, nv));
    }
    if (resplit) launch_mixed_split(ctx->st, GroupOne{scene_of(ctx, ctx->parity), ctx->form}, resplit);
    CK(cudaGetLastError());
    return SPHNJ_OK;
}

}  // namespace

extern "C" {

int sphnj_upload_fields(sphnj_ctx *ctx, uint32_t mask, const sphnj_host_state *s) {
    if (!ctx || !s) return SPHNJ_ERR_ARG;
    if (!ctx->uploaded) return fail(ctx, SPHNJ_ERR_ARG, "sphnj_upload_fields before sphnj_upload");
    cudaSetDevice(ctx->device);
    RET(upload_fields_enqueue(ctx, mask, s, 0u));
    CK(cudaStreamSynchronize(ctx->st));
    return SPHNJ_OK;
}

int sphnj_set_tiling(sphnj_ctx *ctx, int tiled, int tile_h) {
    if (!ctx || tile_h < 1 || tile_h > 64) return SPHNJ_ERR_ARG;
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->st));
    ctx->tiles.tiled = tiled != 0;
    ctx->tiles.tile_h = tile_h;
    drop_graphs(ctx);
    CK(configure_sweeps(ctx->tiles));
    return SPHNJ_OK;
}

int sphnj_diagnostics(sphnj_ctx *ctx, sphnj_diag *out) {
    if (!ctx || !out) return SPHNJ_ERR_ARG;
    if (!ctx->uploaded) return fail(ctx, SPHNJ_ERR_ARG, "sphnj_diagnostics before sphnj_upload");
    cudaSetDevice(ctx->device);
    launch_diagnostics(ctx->st, GroupOne{scene_of(ctx, ctx->parity), ctx->form}, ctx->diag_part, ctx->step,
                       ctx->diag_out);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, ctx->diag_out, sizeof(sphnj_diag), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return check_device_error(ctx);
}

int sphnj_probe(sphnj_ctx *ctx, int n, const float *xy, float *out) {
    if (!ctx || n < 0 || (n > 0 && (!xy || !out))) return SPHNJ_ERR_ARG;
    if (!ctx->uploaded) return fail(ctx, SPHNJ_ERR_ARG, "sphnj_probe before sphnj_upload");
    if (n == 0) return SPHNJ_OK;
    cudaSetDevice(ctx->device);
    if (n > ctx->probe_cap) {
        CK(cudaStreamSynchronize(ctx->st));
        if (ctx->probe_buf) cudaFree(ctx->probe_buf);
        ctx->probe_buf = nullptr;
        ctx->probe_cap = 0;
        CK(cudaMalloc(&ctx->probe_buf, (size_t)n * (sizeof(float2) + sizeof(float4))));
        ctx->probe_cap = n;
    }
    float4 *d_out = static_cast<float4 *>(ctx->probe_buf);
    float2 *d_pts = reinterpret_cast<float2 *>(d_out + ctx->probe_cap);
    CK(cudaMemcpyAsync(d_pts, xy, sizeof(float2) * n, cudaMemcpyHostToDevice, ctx->st));
    launch_probe(ctx->st, GroupOne{scene_of(ctx, ctx->parity), ctx->form}, n, d_pts, d_out);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, d_out, sizeof(float4) * n, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return SPHNJ_OK;
}

int sphnj_set_neighbour_lists(sphnj_ctx *ctx, int on) {
    if (!ctx) return SPHNJ_ERR_ARG;
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->st));
    ctx->tiles.lists = on != 0;
    drop_graphs(ctx);  // the pair pass takes the switch as a launch argument
    return SPHNJ_OK;
}

int sphnj_set_block_sizes(sphnj_ctx *ctx, int shift_threads, int pair_threads) {
    if (!ctx) return SPHNJ_ERR_ARG;
    if (!(shift_threads == 0 || shift_threads == 64 || shift_threads == 128 || shift_threads == 256) ||
        !(pair_threads == 0 || pair_threads == 128 || pair_threads == 256))
        return fail(ctx, SPHNJ_ERR_ARG, "block sizes: shifting pass 0, 64, 128 or 256; pair pass 0, 128 or 256");
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->st));
    ctx->tiles.shift_block = shift_threads;
    ctx->tiles.pair_block = pair_threads;
    drop_graphs(ctx);
    return SPHNJ_OK;
}

int sphnj_get_block_sizes(const sphnj_ctx *ctx, int *shift_threads, int *pair_threads) {
    if (!ctx) return SPHNJ_ERR_ARG;
    if (shift_threads) *shift_threads = ctx->tiles.shift_block;
    if (pair_threads) *pair_threads = ctx->tiles.pair_block;
    return SPHNJ_OK;
}

int sphnj_get_sweeps(const sphnj_ctx *ctx, int *tiled, int *tile_h, int *lists) {
    if (!ctx) return SPHNJ_ERR_ARG;
    if (tiled) *tiled = ctx->tiles.tiled ? 1 : 0;
    if (tile_h) *tile_h = ctx->tiles.tile_h;
    if (lists) *lists = ctx->tiles.lists ? 1 : 0;
    return SPHNJ_OK;
}

int sphnj_profile_stage_count(void) { return ST_COUNT; }
const char *sphnj_profile_stage_name(int s) { return s >= 0 && s < ST_COUNT ? kStageNames[s] : ""; }

int sphnj_profile_enable(sphnj_ctx *ctx, int on) {
    if (!ctx) return SPHNJ_ERR_ARG;
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->st));
    ctx->prof.enable(on != 0);
    return SPHNJ_OK;
}

int sphnj_profile_read(sphnj_ctx *ctx, double *ms, int64_t *calls, int64_t *kernels) {
    if (!ctx) return SPHNJ_ERR_ARG;
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->st));
    CK(ctx->prof.collect());
    for (int s = 0; s < ST_COUNT; ++s) {
        if (ms) ms[s] = ctx->prof.ms[s];
        if (calls) calls[s] = ctx->prof.calls[s];
        if (kernels) kernels[s] = ctx->prof.kernels[s];
    }
    return SPHNJ_OK;
}

int sphnj_stat_launches(const sphnj_ctx *ctx, uint64_t *launches) {
    if (!ctx || !launches) return SPHNJ_ERR_ARG;
    *launches = ctx->launches;
    return SPHNJ_OK;
}

int sphnj_synchronize(sphnj_ctx *ctx) {
    if (!ctx) return SPHNJ_ERR_ARG;
    cudaSetDevice(ctx->device);
    return check_device_error(ctx);
}

}  // extern "C"

namespace {

// sphnj_download without the final device-error check; the fluid densities
// and pressures in `defer` are left out (the caller moves them).
int download_enqueue(sphnj_ctx *ctx, uint32_t mask, sphnj_host_state *s, uint32_t defer) {
    const sphnj_params &p = ctx->p;
    const int nf = p.fluid_number_total, ns = p.solid_number, nv = p.virt_number;
    const DevState &d = ctx->d;
    // fluid fields in device-mapped host memory: one kernel, no copies
    FluidHost fh = fluid_host(mask, s, nf);
    if (defer & DEF_RHO) fh.rho = nullptr;
    if (defer & DEF_P) fh.p = nullptr;
    // mixed form: absolute positions and FP64 solid kinematics from the state
    if (ctx->form == SPHNJ_FORM_MIXED)
        launch_mixed_join(ctx->st, GroupOne{scene_of(ctx, ctx->parity), ctx->form},
                          ((mask & SPHNJ_F_FLUID_KINEMATICS) && !fh.pos ? 1 : 0) |
                              ((mask & (SPHNJ_F_SOLID_KINEMATICS | SPHNJ_F_SOLID_DERIVED)) ? 2 : 0));
    launch_fluid_to_host(ctx->st, GroupOne{scene_of(ctx, ctx->parity), ctx->form}, fh);
    if (mask & SPHNJ_F_FLUID_KINEMATICS) {
        if (!fh.pos) RET(d2h(ctx, s->fluid_position, d.f_pos, nf));
        if (!fh.vel) RET(d2h(ctx, s->fluid_velocity, d.f_vel, nf));
    }
    if (mask & SPHNJ_F_FLUID_THERMO) {
        if (!fh.rho && !(defer & DEF_RHO)) RET(d2h(ctx, s->fluid_density, d.f_rho, nf));
        if (!fh.p && !(defer & DEF_P)) RET(d2h(ctx, s->fluid_pressure, d.f_p, nf));
        RET(enum_d2h(ctx, s->fluid_phase, d.f_phase, nf));
    }
    if (mask & SPHNJ_F_FLUID_FLAGS) {
        RET(enum_d2h(ctx, s->fluid_boundary_type, d.f_fbt, nf));
        RET(enum_d2h(ctx, s->fluid_has_near_particle, d.f_near, nf));
    }
    if (mask & SPHNJ_F_FLUID_DERIVED) {
        RET(d2h(ctx, s->fluid_du_dx, d.f_dudx, nf));
        RET(d2h(ctx, s->fluid_gradient, d.f_grad, nf));
        RET(d2h(ctx, s->fluid_du_dt, d.f_dudt, nf));
        RET(d2h(ctx, s->fluid_color, d.f_color, nf));
        RET(d2h(ctx, s->fluid_drho_dt, d.f_drho, nf));
    }
    if (mask & SPHNJ_F_SOLID_KINEMATICS) {
        RET(d2h(ctx, s->solid_position, d.s_pos, ns));
        RET(d2h(ctx, s->solid_reference_position, d.s_ref, ns));
        RET(d2h(ctx, s->solid_velocity, d.s_vel, ns));
    }
    if (mask & SPHNJ_F_SOLID_MATERIAL) {
        RET(enum_d2h(ctx, s->solid_boundary_type, d.s_bt, ns));
        RET(enum_d2h(ctx, s->solid_material_type, d.s_mat, ns));
        RET(d2h(ctx, s->solid_max_strain, d.s_maxstrain, ns));
    }
    if (mask & SPHNJ_F_SOLID_DERIVED) {
        RET(d2h(ctx, s->solid_pressure, d.s_p, ns));
        RET(d2h(ctx, s->solid_deformation, d.s_F, ns));
        RET(d2h(ctx, s->solid_stress_1st_piola, d.s_P, ns));
        RET(d2h(ctx, s->solid_correction, d.s_L, ns));
        RET(d2h(ctx, s->solid_du_dt, d.s_dudt, ns));
        RET(d2h(ctx, s->solid_normal, d.s_normal, ns));
        RET(d2h(ctx, s->solid_couple_dudt, d.s_couple, ns));
    }
    if (mask & SPHNJ_F_VIRT) {
        RET(d2h(ctx, s->virt_position, d.v_pos, nv));
        RET(d2h(ctx, s->virt_normal, d.v_normal, nv));
        RET(d2h(ctx, s->virt_velocity, d.v_vel, nv));
        RET(d2h(ctx, s->virt_pressure, d.v_p, nv));
        RET(d2h(ctx, s->virt_density, d.v_rho, nv));
        RET(enum_d2h(ctx, s->virt_phase, d.v_phase, nv));
        RET(enum_d2h(ctx, s->virt_boundary_type, d.v_bt, nv));
    }
    if (mask & SPHNJ_F_CELL_IDS) {
        RET(d2h(ctx, s->fluid_cell_id, d.f_cell, nf));
        RET(d2h(ctx, s->solid_cell_id, d.s_cell, ns));
        RET(d2h(ctx, s->virt_cell_id, d.v_cell, nv));
    }
    return SPHNJ_OK;
}

}  // namespace

extern "C" {

int sphnj_download(sphnj_ctx *ctx, uint32_t mask, sphnj_host_state *s) {
    if (!ctx || !s) return SPHNJ_ERR_ARG;
    cudaSetDevice(ctx->device);
    RET(download_enqueue(ctx, mask, s, 0u));
    return check_device_error(ctx);
}

int sphnj_step_exchange(sphnj_ctx *ctx, int n, uint32_t in_mask, const sphnj_host_state *in, uint32_t out_mask,
                        sphnj_host_state *out) {
    if (!ctx || n < 1) return SPHNJ_ERR_ARG;
    if (!ctx->uploaded) return fail(ctx, SPHNJ_ERR_ARG, "sphnj_step_exchange before sphnj_upload");
    if (ctx->batch) return fail(ctx, SPHNJ_ERR_ARG, "the scene is in a batch: step the batch");
    cudaSetDevice(ctx->device);
    const int nf = ctx->p.fluid_number_total;
    const DevState &d = ctx->d;
    if (!ctx->io_st) {
        if (cudaStreamCreateWithFlags(&ctx->io_st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_start, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_in, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_rho_p, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_out, cudaEventDisableTiming) != cudaSuccess)
            return cuda_fail(ctx, cudaGetLastError(), "step_exchange streams");
    }
    cudaStream_t st = ctx->st, io = ctx->io_st;
    // Fluid velocities, densities and pressures go up on the second stream,
    // after everything queued so far, while the first step bins and builds
    // its lists; its first stage that reads them waits (StepKind::io bit 0).
    uint32_t in_late = 0;
    if (in && nf > 0) {
        if ((in_mask & SPHNJ_F_FLUID_KINEMATICS) && in->fluid_velocity) in_late |= DEF_VEL;
        if ((in_mask & SPHNJ_F_FLUID_THERMO) && in->fluid_density) in_late |= DEF_RHO;
        if ((in_mask & SPHNJ_F_FLUID_THERMO) && in->fluid_pressure) in_late |= DEF_P;
    }
    // The last step's densities and pressures come down on the second stream
    // during its shifting passes (after the fluid update, StepKind::io bit 1).
    uint32_t out_late = 0;
    if (out && nf > 0 && (out_mask & SPHNJ_F_FLUID_THERMO)) {
        if (out->fluid_density) out_late |= DEF_RHO;
        if (out->fluid_pressure) out_late |= DEF_P;
    }
    const size_t n2 = sizeof(float2) * (size_t)nf, n1 = sizeof(float) * (size_t)nf;
    if (in_late) {
        CK(cudaEventRecord(ctx->ev_start, st));
        CK(cudaStreamWaitEvent(io, ctx->ev_start, 0));
        if (in_late & DEF_VEL) CK(cudaMemcpyAsync(d.f_vel, in->fluid_velocity, n2, cudaMemcpyHostToDevice, io));
        if (in_late & DEF_RHO) CK(cudaMemcpyAsync(d.f_rho, in->fluid_density, n1, cudaMemcpyHostToDevice, io));
        if (in_late & DEF_P) CK(cudaMemcpyAsync(d.f_p, in->fluid_pressure, n1, cudaMemcpyHostToDevice, io));
        CK(cudaEventRecord(ctx->ev_in, io));
    }
    if (in) RET(upload_fields_enqueue(ctx, in_mask, in, in_late));
    RET(run_steps(ctx, n, in_late ? 1 : 0, out_late ? 2 : 0));
    if (out_late) {
        CK(cudaStreamWaitEvent(io, ctx->ev_rho_p, 0));
        if (out_late & DEF_RHO) CK(cudaMemcpyAsync(out->fluid_density, d.f_rho, n1, cudaMemcpyDeviceToHost, io));
        if (out_late & DEF_P) CK(cudaMemcpyAsync(out->fluid_pressure, d.f_p, n1, cudaMemcpyDeviceToHost, io));
        CK(cudaEventRecord(ctx->ev_out, io));
    }
    if (out) RET(download_enqueue(ctx, out_mask, out, out_late));
    if (out_late) CK(cudaStreamWaitEvent(st, ctx->ev_out, 0));
    return check_device_error(ctx);
}

int sphnj_get_step(const sphnj_ctx *ctx, int *step) {
    if (!ctx || !step) return SPHNJ_ERR_ARG;
    *step = ctx->step;
    return SPHNJ_OK;
}

int sphnj_debug_cells(sphnj_ctx *ctx, int type, int32_t *start, int32_t *count, int32_t *list, int32_t *n_listed) {
    if (!ctx || type < 0 || type > 2) return SPHNJ_ERR_ARG;
    cudaSetDevice(ctx->device);
    const int C = ctx->p.cell_number_total;
    const CellList &L = type == 0 ? ctx->lf[ctx->parity] : type == 1 ? ctx->ls[ctx->parity] : ctx->lv;
    const int n = type == 0 ? ctx->p.fluid_number_total : type == 1 ? ctx->p.solid_number : ctx->p.virt_number;
    int2 *h = new int2[C > 0 ? C : 1];
    cudaError_t e = cudaMemcpyAsync(h, L.rng, sizeof(int2) * C, cudaMemcpyDeviceToHost, ctx->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
    if (e != cudaSuccess) {
        delete[] h;
        return cuda_fail(ctx, e, "debug_cells");
    }
    int total = 0;
    for (int c = 0; c < C; ++c) {
        if (start) start[c] = h[c].x;
        if (count) count[c] = h[c].y;
        total += h[c].y;
    }
    delete[] h;
    if (n_listed) *n_listed = total;
    if (list && total > 0 && total <= n) {
        CK(cudaMemcpyAsync(list, L.lst, sizeof(int) * total, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    return check_device_error(ctx);
}

int sphnj_debug_set_cells(sphnj_ctx *ctx, const int32_t *cf, const int32_t *lf, const int32_t *cs,
                          const int32_t *ls, const int32_t *cv, const int32_t *lv) {
    if (!ctx) return SPHNJ_ERR_ARG;
    cudaSetDevice(ctx->device);
    const int C = ctx->p.cell_number_total;
    const int ns_[3] = {ctx->p.fluid_number_total, ctx->p.solid_number, ctx->p.virt_number};
    const int32_t *cnt[3] = {cf, cs, cv}, *lst[3] = {lf, ls, lv};
    CellList L[3] = {ctx->lf[ctx->parity], ctx->ls[ctx->parity], ctx->lv};
    int2 *h = new int2[C > 0 ? C : 1];
    long listed[3] = {0, 0, 0};
    for (int k = 0; k < 3; ++k) {
        long acc = 0;
        for (int c = 0; c < C; ++c) {
            int n = cnt[k] ? cnt[k][c] : 0;
            h[c] = make_int2((int)acc, n);
            acc += n;
        }
        listed[k] = acc;
        if (acc > ns_[k] || (acc > 0 && !lst[k])) {
            delete[] h;
            return fail(ctx, SPHNJ_ERR_ARG, "debug_set_cells: list longer than the particle count");
        }
        for (long q = 0; q < acc; ++q)
            if (lst[k][q] < 0 || lst[k][q] >= ns_[k]) {
                delete[] h;
                return fail(ctx, SPHNJ_ERR_ARG, "debug_set_cells: particle index out of range");
            }
        cudaError_t e = cudaMemcpyAsync(L[k].rng, h, sizeof(int2) * C, cudaMemcpyHostToDevice, ctx->st);
        if (e == cudaSuccess && acc > 0)
            e = cudaMemcpyAsync(L[k].lst, lst[k], sizeof(int) * acc, cudaMemcpyHostToDevice, ctx->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
        if (e != cudaSuccess) {
            delete[] h;
            return cuda_fail(ctx, e, "debug_set_cells");
        }
    }
    delete[] h;
    // virtual lists that hold every virtual particle mean the first sort
    // already happened (their order and ids are final)
    ctx->virt_sorted = ns_[2] > 0 && listed[2] == ns_[2];
    bind_lists(ctx);
    return SPHNJ_OK;
}

int sphnj_debug_set_step(sphnj_ctx *ctx, int step) {
    if (!ctx) return SPHNJ_ERR_ARG;
    ctx->step = step;
    return SPHNJ_OK;
}

int sphnj_debug_max_speed(sphnj_ctx *ctx, float *ms) {
    if (!ctx || !ms) return SPHNJ_ERR_ARG;
    cudaSetDevice(ctx->device);
    unsigned int bits = 0;
    CK(cudaMemcpyAsync(&bits, ctx->d.max_speed2_bits, sizeof bits, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    float v2;
    std::memcpy(&v2, &bits, sizeof v2);
    float vmax = sqrtf(v2);
    float cap = 0.1f * std::min(ctx->p.sound_speed[0], ctx->p.sound_speed[1]);
    *ms = std::min(vmax, cap);
    return SPHNJ_OK;
}

const char *sphnj_last_error(const sphnj_ctx *ctx) { return ctx ? ctx->msg.c_str() : "null context"; }

}  // extern "C"
