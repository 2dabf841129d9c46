// libps3d_gpu.so: the C ABI declared in include/ps3d_gpu.h.
//
// Host orchestration of the GB300 kernels in transforms.cu and ops.cu.  The
// routines follow the reference procedures they replace (cited per
// function); the spectral algebra is regrouped so that every x/y derivative
// is an in-register coefficient times a partner column and every
// combine/scale/decompose sandwich of the steppers becomes a bare column
// scaling.  Two precisions share the code through the template parameter T
// (the storage type of every transient field): FP64, and mixed (FP32
// transient fields with FP64 prognostic vorticity, RK accumulators,
// low-mode inversion and reductions).
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ps3d_gpu.h"
#include "kernels.h"

using namespace ps3d;

namespace {

constexpr int NTMP = 6;


struct Rolling {
    std::vector<double> hist;
    int inew = 1, iold = 1;
    bool filled = false;
    double sma = 0.0;
    // rolling_mean_t%get_next (rolling_mean.f90:36-69)
    double next(double v)
    {
        const int L = (int)hist.size();
        if (filled) {
            const double vold = hist[iold - 1];
            iold = iold % L + 1;
            sma = sma + (v - vold) / (double)L;
            hist[inew - 1] = v;
            inew = inew % L + 1;
        } else {
            hist[inew - 1] = v;
            double s = 0.0;
            for (int i = 0; i < inew; ++i) s += hist[i];
            sma = s / (double)inew;
            filled = (L == inew);
            inew = inew % L + 1;
        }
        return sma;
    }
};

// Per-step scalars in device memory.  The mixed stage kernels read dt here;
// in a captured step (CUDA graph) adapt's scalar logic also runs on the
// device and leaves the step's diagnostics here.
struct StepScal {
    double dt;         // time step of the current step
    double t;          // model time at the start of the next step
    double dfac;       // diffusion factor of vdiss (impl-diff-rk4: pref dt / 2)
    double diag[22];   // ps3d_gpu_diag of the last step, field by field
    double sma;        // rolling mean of the strain maximum (rolling_mean.f90)
    int inew, iold, filled;
    int err;           // 1 non-finite diagnostic, 2 Jacobi sweep limit
};

struct BatchPlan;

}  // namespace

struct ps3d_gpu_ctx {
    ps3d_gpu_config cfg;
    Dims d;
    bool fp64 = true;
    // mixed source: products formed inside their forward y-line kernel
    // (set at creation, see products_fused_default)
    bool fuse_products = false;
    // advance_host's state check on a second stream beside the first
    // right-hand side (mixed form): staging array svorf, flag_chk, resolved
    // by advance before the stage updates
    cudaStream_t st_chk = nullptr;
    cudaEvent_t ev_chk0 = nullptr, ev_chk = nullptr;
    int *flag_chk = nullptr;
    bool pending_check = false;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    long long launches = 0;
    long long bytes = 0;
    std::vector<void *> allocs;

    // FP64 prognostic state and RK accumulators
    double *svor = nullptr, *svori = nullptr, *svorf = nullptr, *vortsm = nullptr;
    double *stage64 = nullptr;   // FP64 staging field for mixed-precision transfers
    float *svor32 = nullptr;     // FP32 copy of svor read by the mixed vor2vel
    // mixed form: es = decompose(diffz(svorts(3))), the z part of the
    // tendency's solenoidal projection, left by source for the fused stage
    // update; the FP64 (0,0) column of the current stage state (components
    // 1 and 2, pitch P), read by the mean-flow inversion while the FP64
    // state still holds the step's initial state (mf_a: where vor2vel reads
    // that column from; null = svor itself)
    float *es_src = nullptr;
    double *mf64 = nullptr;
    const double *mf_a = nullptr;
    // transient fields (storage type T)
    void *vor = nullptr, *vel = nullptr, *svel = nullptr, *svorts = nullptr, *held = nullptr;
    void *tmp = nullptr;         // NTMP consecutive fields
    void *phim = nullptr, *phip = nullptr, *thetam = nullptr, *thetap = nullptr, *dthetam = nullptr,
         *dthetap = nullptr, *green = nullptr;
    void *twx = nullptr, *twy = nullptr, *twz2 = nullptr;
    // FP32 z-transform tables of the mixed form: exp(-2 pi i k/nz), sin and
    // cos(j pi/nz)
    float2 *twz32 = nullptr;
    float *sinz32 = nullptr, *cosz32 = nullptr;
    // FP64 transform tables for the FP64 set-up / projection of the mixed
    // form (aliases of the above in the FP64 form)
    double2 *twx64 = nullptr, *twy64 = nullptr, *twz2_64 = nullptr;
    double *phim64 = nullptr, *phip64 = nullptr;
    // per-column and per-level FP64 tables
    double *k2l2 = nullptr, *k2l2i = nullptr, *filt0 = nullptr, *vhdis = nullptr, *vdiss = nullptr;
    double *epq = nullptr, *emq = nullptr, *epq2 = nullptr, *emq2 = nullptr;
    double *fz = nullptr, *rkz = nullptr, *rkzi = nullptr, *gamtop = nullptr, *gambot = nullptr;
    double *dstsum = nullptr, *dctcos = nullptr, *cx = nullptr, *cy = nullptr, *zm = nullptr, *zp = nullptr;
    double *ubar = nullptr, *vbar = nullptr, *ini = nullptr, *savg = nullptr;
    double *part = nullptr, *res1 = nullptr, *res2 = nullptr;
    int *flag = nullptr;
    // host copies
    std::vector<double> h_rkx, h_rky, h_rkz, h_k2l2, h_k2l2i, h_filt0, h_fz, h_gamtop, h_gambot;
    double dx[3], ncelli, fnzi, dzi;
    long long ncell;
    double vvisc = 0.0;
    bool diffusion_ready = false;
    double ini_vor_mean[2] = {0.0, 0.0};
    Rolling roll;
    Probe probe;
    // device-side step scalars, rolling-mean history, captured step
    StepScal *sc = nullptr;
    double *roll_dev = nullptr;
    cudaGraphExec_t graph = nullptr;
    long long graph_launches = 0;  // kernels per captured step
    // the captured batch step this context leads (ps3d_gpu_batch_advance),
    // and the serial number that identifies the context in another's batch
    BatchPlan *batch = nullptr;
    unsigned long long serial = 0;
    // line-FFT autotuner: ms per launch of each kernel shape for the passes
    // forward y, forward x, inverse y, inverse x (0 where not timed)
    double tune_ms[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    // kinetic-energy spectrum scratch (allocated on first use): rkx, rky,
    // shell sums, shell counts
    double *spec_buf = nullptr;
    int spec_kmax = -1;
    // buoyancy (the reference's ENABLE_BUOYANCY build): the FP64 state b'
    // (mixed-spectral) with its RK accumulators (sbuoyf holds FP32
    // increments in the mixed form) and cn2 predictor, the FP32 copy read by
    // the mixed form, transient fields of type T, per-column factors
    double *sbuoy = nullptr, *sbuoyi = nullptr, *sbuoyf = nullptr, *bsm = nullptr;
    float *sbuoy32 = nullptr;
    void *buoy = nullptr, *sbuoys = nullptr, *heldb = nullptr, *dphim = nullptr, *dphip = nullptr;
    double *bhdis = nullptr, *bdiss = nullptr, *bpq = nullptr, *bmq = nullptr, *bpq2 = nullptr, *bmq2 = nullptr;
    double *bpart = nullptr, *bres = nullptr, *bprof = nullptr;
    unsigned long long *bmax = nullptr;
    std::vector<double> h_bbarz;
    double bfsq = 0.0, bvisc = 0.0;
    Rolling roll_b;
    // learned sub-grid closure (closure.cu): the attached network, its
    // correction (3 fields of type T in the form svorts is assembled in)
    // and whether the next source evaluates it afresh
    ps3d_closure *closure = nullptr;
    void *corr = nullptr;
    int closure_flags = 0;  // PS3D_CLOSURE_*
    bool closure_fresh = true;

    Deriv D() const { return Deriv{cx, cy}; }
    Tables tables() const
    {
        return Tables{k2l2i, filt0, vhdis, epq, emq, epq2, emq2, vdiss, fz, rkz, rkzi, gamtop, gambot, dstsum,
                      dctcos};
    }
};

namespace {

int fail(ps3d_gpu_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

int check(ps3d_gpu_ctx *c, const char *where)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, PS3D_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
    return PS3D_OK;
}

int sync_check(ps3d_gpu_ctx *c, const char *where)
{
    cudaError_t e = cudaStreamSynchronize(c->st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, PS3D_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
    return PS3D_OK;
}

template <typename P> bool dalloc(ps3d_gpu_ctx *c, P **p, size_t bytes)
{
    void *q = nullptr;
    if (cudaMalloc(&q, bytes) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaMemsetAsync(q, 0, bytes, c->st);
    c->allocs.push_back(q);
    c->bytes += (long long)bytes;
    *p = (P *)q;
    return true;
}

template <typename T> T *tf(void *p) { return reinterpret_cast<T *>(p); }
template <typename T> T *tmpf(ps3d_gpu_ctx *c, int i) { return tf<T>(c->tmp) + (size_t)i * c->d.nfield; }
template <typename T> using CT = typename cplx<T>::type;

// launch-count bookkeeping (kernels per host-side operation)
constexpr int NL_COL = 1;

// ---------------------------------------------------------------- transfers
// host (nz+1)-pitched columns <-> device P-pitched columns
int upload(ps3d_gpu_ctx *c, const double *h, int ncomp, void *dst, bool dst_is_fp64)
{
    const Dims &d = c->d;
    const size_t hp = (size_t)(d.nz + 1) * sizeof(double);
    for (int k = 0; k < ncomp; ++k) {
        const double *hk = h + (size_t)k * (d.nz + 1) * d.ncol;
        if (dst_is_fp64) {
            double *dk = tf<double>(dst) + (size_t)k * d.nfield;
            if (cudaMemcpy2DAsync(dk, d.P * sizeof(double), hk, hp, hp, d.ncol, cudaMemcpyHostToDevice, c->st) !=
                cudaSuccess)
                return check(c, "upload");
        } else {
            if (cudaMemcpy2DAsync(c->stage64, d.P * sizeof(double), hk, hp, hp, d.ncol, cudaMemcpyHostToDevice,
                                  c->st) != cudaSuccess)
                return check(c, "upload");
            op_convert<float, double>(d, c->st, c->stage64, tf<float>(dst) + (size_t)k * d.nfield, d.nfield);
            c->launches += 1;
        }
    }
    return check(c, "upload");
}

int download(ps3d_gpu_ctx *c, const void *src, bool src_is_fp64, int ncomp, double *h)
{
    const Dims &d = c->d;
    const size_t hp = (size_t)(d.nz + 1) * sizeof(double);
    for (int k = 0; k < ncomp; ++k) {
        double *hk = h + (size_t)k * (d.nz + 1) * d.ncol;
        const double *sk;
        if (src_is_fp64) {
            sk = tf<const double>(const_cast<void *>(src)) + (size_t)k * d.nfield;
        } else {
            op_convert<double, float>(d, c->st, tf<const float>(const_cast<void *>(src)) + (size_t)k * d.nfield,
                                      c->stage64, d.nfield);
            c->launches += 1;
            sk = c->stage64;
        }
        if (cudaMemcpy2DAsync(hk, hp, sk, d.P * sizeof(double), hp, d.ncol, cudaMemcpyDeviceToHost, c->st) !=
            cudaSuccess)
            return check(c, "download");
    }
    return sync_check(c, "download");
}

// ------------------------------------------------------------- primitives
// launches of one line pass over nf fields: one for the FP32 line kernels,
// one per field otherwise
template <typename T> int line_launches(const ps3d_gpu_ctx *c, int n, int nf)
{
    return (sizeof(T) == sizeof(float) && lines32_supported(n)) ? 1 : nf;
}
// horizontal transforms of nf consecutive fields (nfield apart)
template <typename T> void xyf(ps3d_gpu_ctx *c, const T *in, T *out, int nf = 1)
{
    xy_forward<T>(c->d, c->st, in, out, tf<CT<T>>(c->twx), tf<CT<T>>(c->twy), &c->probe, nf);
    c->launches += line_launches<T>(c, c->d.ny, nf) + line_launches<T>(c, c->d.nx, nf);
}
template <typename T> void xyi(ps3d_gpu_ctx *c, const T *in, T *out, int nf = 1)
{
    xy_inverse<T>(c->d, c->st, in, out, tf<CT<T>>(c->twx), tf<CT<T>>(c->twy), &c->probe, nf);
    c->launches += line_launches<T>(c, c->d.ny, nf) + line_launches<T>(c, c->d.nx, nf);
}
template <typename T, typename TIN> void col_any(ps3d_gpu_ctx *c, int mode, const TIN *in, T *out)
{
    if (sizeof(T) == sizeof(float) && colz_supported(c->d.nz)) {
        columns_z<TIN>(c->d, c->st, mode, in, reinterpret_cast<float *>(out), c->k2l2, (float)c->dx[2],
                       (float)c->cfg.extent[2], c->twz32, c->sinz32, c->cosz32, &c->probe);
    } else if (sizeof(T) == sizeof(float) && col32_supported(c->d.nz)) {
        columns32<TIN>(c->d, c->st, mode, in, reinterpret_cast<float *>(out), c->k2l2, (float)c->dx[2],
                       (float)c->cfg.extent[2], tf<float2>(c->twz2), &c->probe);
    } else if (sizeof(TIN) == sizeof(T)) {
        columns<T>(c->d, c->st, mode, reinterpret_cast<const T *>(in), out, tf<T>(c->phim), tf<T>(c->phip),
                   tf<CT<T>>(c->twz2), &c->probe);
    } else {
        columns_in<float, double>(c->d, c->st, mode, reinterpret_cast<const double *>(in),
                                  reinterpret_cast<float *>(out), tf<float>(c->phim), tf<float>(c->phip),
                                  tf<float2>(c->twz2), &c->probe);
    }
    c->launches += NL_COL;
}
template <typename T> void col(ps3d_gpu_ctx *c, int mode, const T *in, T *out) { col_any<T, T>(c, mode, in, out); }
// a T view of an FP64 state component (copy for the mixed form)
template <typename T> const T *state_as_T(ps3d_gpu_ctx *c, const double *s, T *scratch)
{
    if (sizeof(T) == sizeof(double)) return reinterpret_cast<const T *>(s);
    op_convert<float, double>(c->d, c->st, s, reinterpret_cast<float *>(scratch), c->d.nfield);
    c->launches += 1;
    return scratch;
}
template <typename T> void state_from_T(ps3d_gpu_ctx *c, const T *src, double *s)
{
    if (sizeof(T) == sizeof(double)) {
        if ((const void *)src != (const void *)s)
            cudaMemcpyAsync(s, src, c->d.nfield * sizeof(double), cudaMemcpyDeviceToDevice, c->st);
        return;
    }
    op_convert<double, float>(c->d, c->st, reinterpret_cast<const float *>(src), s, c->d.nfield);
    c->launches += 1;
}

// FP64 scratch fields for the FP64 projection: the FP64 form uses its
// transient temporaries, the mixed form the RK accumulator svorf (free
// outside a step)
double *scratch64(ps3d_gpu_ctx *c, int i)
{
    if (c->fp64) return tmpf<double>(c, i);
    return c->svorf + (size_t)i * c->d.nfield;
}

// Solenoidal projection of the prognostic vorticity in FP64
// (inversion.f90:34-76): ds = B_x - A_y, es = decompose(diffz(combine(C))),
// A = k2l2i (es_x + ds_y), B = k2l2i (es_y - ds_x), (0,0) column kept.
void project64(ps3d_gpu_ctx *c)
{
    const Dims &d = c->d;
    const long long N = d.nfield;
    double *A = c->svor, *B = c->svor + N, *Cc = c->svor + 2 * N;
    double *cs = scratch64(c, 0), *es = scratch64(c, 1), *ds = scratch64(c, 2);
    op_v2v_ds<double, double>(d, c->st, c->D(), A, B, ds);
    columns<double>(d, c->st, COL_COMBINE, Cc, cs, c->phim64, c->phip64, c->twz2_64, nullptr);
    op_diffz<double>(d, c->st, c->dzi, cs, es);
    columns<double>(d, c->st, COL_DECOMP, es, es, c->phim64, c->phip64, c->twz2_64, nullptr);
    op_v2v_project<double, double>(d, c->st, c->D(), c->k2l2i, es, ds, A, B);
    c->launches += 5;
}

// FP32 copy of the prognostic state for the mixed form's vor2vel
void refresh32(ps3d_gpu_ctx *c)
{
    if (c->fp64) return;
    op_narrow(c->st, c->svor, c->svor32, 3 * c->d.nfield);
    c->launches += 1;
}

// projection of an externally set state, then its FP32 copy (mixed form)
void project_state_mixed(ps3d_gpu_ctx *c)
{
    project64(c);
    refresh32(c);
}

// ------------------------------------------------------------------ vor2vel
// inversion.f90:23-226.  The FP64 form follows the reference: the
// solenoidal projection of svor, then the physical vorticity and the
// velocity.  The mixed form keeps svor solenoidal by construction instead
// (svor is projected in FP64 whenever it is set from outside, and every
// source term is projected before the stage update; the projection is
// linear and commutes with the per-column integrating factors, so the
// projected trajectory is the reference's), which keeps FP32 rounding out of
// the prognostic state; vor2vel then only evaluates vor, vel and svel.
template <typename T> int vor2vel_mixed(ps3d_gpu_ctx *c);

template <typename T> int vor2vel(ps3d_gpu_ctx *c)
{
    if (sizeof(T) == sizeof(float)) return vor2vel_mixed<T>(c);
    const Dims &d = c->d;
    const long long N = d.nfield;
    double *A = c->svor, *B = c->svor + N, *Cc = c->svor + 2 * N;
    T *cs = tmpf<T>(c, 0), *es = tmpf<T>(c, 1), *ds = tmpf<T>(c, 2), *bs = tmpf<T>(c, 3), *dsg = tmpf<T>(c, 4),
      *as = tmpf<T>(c, 5);
    T *vor = tf<T>(c->vor), *vel = tf<T>(c->vel), *svel = tf<T>(c->svel);
    const Deriv D = c->D();

    // solenoidal projection (inversion.f90:34-76)
    op_v2v_ds<T, double>(d, c->st, D, A, B, ds);
    col<T>(c, COL_COMBINE, state_as_T<T>(c, Cc, bs), cs);
    op_diffz<T>(d, c->st, c->dzi, cs, es);
    col<T>(c, COL_DECOMP, es, es);
    op_v2v_project<T, double>(d, c->st, D, c->k2l2i, es, ds, A, B);
    c->launches += 3;

    // vorticity in physical space (field_combine_physical x3, :80-82)
    col<T>(c, COL_COMBINE, state_as_T<T>(c, A, bs), bs);
    xyi<T>(c, bs, vor);
    col<T>(c, COL_COMBINE, state_as_T<T>(c, B, bs), bs);
    xyi<T>(c, bs, vor + N);
    xyi<T>(c, cs, vor + 2 * N);

    // vertical velocity (:86-139)
    op_v2v_wsrc<T, double>(d, c->st, D, A, B, ds);
    op_v2v_wprep<T>(d, c->st, ds, tf<T>(c->thetam), tf<T>(c->thetap), tf<T>(c->dthetam), tf<T>(c->dthetap),
                    tf<T>(c->green), c->rkz, bs, es, dsg, as);
    col<T>(c, COL_DCT, as, as);
    col<T>(c, COL_DST, dsg, dsg);
    op_v2v_wfinish<T>(d, c->st, dsg, bs, as, svel + 2 * N, es);
    // mean flow (:150-165) and u, v (:169-213)
    op_v2v_meanflow<double>(d, c->st, A, B, c->tables(), c->ubar, c->vbar);
    op_v2v_uv<T>(d, c->st, D, c->k2l2i, es, cs, c->ubar, c->vbar, svel, svel + N);
    c->launches += 5;
    for (int k = 0; k < 3; ++k) xyi<T>(c, svel + k * N, vel + k * N);
    return check(c, "vor2vel");
}

template <typename T> int vor2vel_mixed(ps3d_gpu_ctx *c)
{
    const Dims &d = c->d;
    const long long N = d.nfield;
    const double *A = c->svor, *B = c->svor + N;
    const T *A32 = reinterpret_cast<const T *>(c->svor32), *B32 = A32 + N, *C32 = A32 + 2 * N;
    T *cs = tmpf<T>(c, 0), *es = tmpf<T>(c, 1), *ds = tmpf<T>(c, 2), *bs = tmpf<T>(c, 3), *dsg = tmpf<T>(c, 4),
      *as = tmpf<T>(c, 5);
    T *vor = tf<T>(c->vor), *vel = tf<T>(c->vel), *svel = tf<T>(c->svel);
    const Deriv D = c->D();
    // vorticity in physical space (field_combine_physical x3) from the FP32
    // copy of the state: the first two components combined straight into
    // vor, the third into cs (which the horizontal inversion reads below);
    // x lines of the first two in place and of the third into vor, then the
    // y lines of all three in one launch
    col<T>(c, COL_COMBINE, A32, vor);
    col<T>(c, COL_COMBINE, B32, vor + N);
    col<T>(c, COL_COMBINE, C32, cs);
    x_inverse<T>(d, c->st, vor, vor, tf<CT<T>>(c->twx), &c->probe, 2);
    x_inverse<T>(d, c->st, cs, vor + 2 * N, tf<CT<T>>(c->twx), &c->probe, 1);
    y_inverse<T>(d, c->st, vor, vor, tf<CT<T>>(c->twy), &c->probe, 3);
    c->launches += line_launches<T>(c, d.nx, 2) + line_launches<T>(c, d.nx, 1) + line_launches<T>(c, d.ny, 3);
    // vertical velocity, mean flow, u, v (inversion.f90:86-213)
    if (columns_w_src_supported(d.nz)) {
        // w and dw/dz in two column kernels that also form the w source ds
        // from the partner columns of the state (ds stays on chip)
        columns_w_src(d, c->st, reinterpret_cast<const float *>(A32), reinterpret_cast<const float *>(B32),
                      reinterpret_cast<float *>(svel + 2 * N), reinterpret_cast<float *>(es), c->k2l2, c->k2l2i,
                      D.cx, D.cy, (float)c->dx[2], (float)c->cfg.extent[2], c->twz32, c->sinz32, c->cosz32,
                      &c->probe);
        c->launches += 2;
    } else if (colz_supported(d.nz)) {
        op_v2v_wsrc<T, T>(d, c->st, D, A32, B32, ds);
        c->launches += 1;
        // w and dw/dz in two column kernels, one per output (theta
        // functions and the Green function evaluated in registers)
        columns_w(d, c->st, reinterpret_cast<const float *>(ds), reinterpret_cast<float *>(svel + 2 * N),
                  reinterpret_cast<float *>(es), c->k2l2, c->k2l2i, (float)c->dx[2], (float)c->cfg.extent[2],
                  c->twz32, c->sinz32, c->cosz32, &c->probe);
        c->launches += 2;
    } else {
        op_v2v_wsrc<T, T>(d, c->st, D, A32, B32, ds);
        op_v2v_wprep<T>(d, c->st, ds, tf<T>(c->thetam), tf<T>(c->thetap), tf<T>(c->dthetam), tf<T>(c->dthetap),
                        tf<T>(c->green), c->rkz, bs, es, dsg, as);
        col<T>(c, COL_DCT, as, as);
        col<T>(c, COL_DST, dsg, dsg);
        op_v2v_wfinish<T>(d, c->st, dsg, bs, as, svel + 2 * N, es);
        c->launches += 3;
    }
    // the (0,0) column of the stage state: FP64 (mf64) inside a step
    const double *mA = c->mf_a ? c->mf_a : A, *mB = c->mf_a ? c->mf_a + d.P : B;
    op_v2v_meanflow<double>(d, c->st, mA, mB, c->tables(), c->ubar, c->vbar);
    op_v2v_uv<T>(d, c->st, D, c->k2l2i, es, cs, c->ubar, c->vbar, svel, svel + N);
    c->launches += 2;
    xyi<T>(c, svel, vel, 3);
    return check(c, "vor2vel");
}

// The tail of the mixed source: the three tendency components decomposed
// (field_decompose_semi_spectral, inversion_utils.f90:614-647) and es =
// decompose(central_diffz(S3)), the z part of the tendency's solenoidal
// projection (inversion.f90:41-47), for the fused stage update.  The
// tendency itself stays unprojected, as the reference's source leaves it.
template <typename T> void source_decompose_mixed(ps3d_gpu_ctx *c)
{
    const Dims &d = c->d;
    const long long N = d.nfield;
    T *S1 = tf<T>(c->svorts), *S2 = S1 + N, *S3 = S1 + 2 * N;
    T *es = reinterpret_cast<T *>(c->es_src);
    col<T>(c, COL_DECOMP, S1, S1);
    col<T>(c, COL_DECOMP, S2, S2);
    if (colz_supported(d.nz)) {
        columns_dec2(d, c->st, reinterpret_cast<const float *>(S3), reinterpret_cast<float *>(S3),
                     reinterpret_cast<float *>(es), c->k2l2, (float)c->dx[2], (float)c->cfg.extent[2], c->twz32,
                     c->sinz32, &c->probe);
        c->launches += 1;
    } else {
        T *g = tmpf<T>(c, 0);
        op_diffz<T>(d, c->st, c->dzi, S3, g);
        c->launches += 1;
        col<T>(c, COL_DECOMP, g, es);
        col<T>(c, COL_DECOMP, S3, S3);
    }
}

// ----------------------------------------------------------------- buoyancy
// The buoyancy state b' as read by the transforms (FP32 copy in the mixed form)
template <typename T> const T *sbuoy_T(ps3d_gpu_ctx *c)
{
    if (sizeof(T) == sizeof(double)) return reinterpret_cast<const T *>(c->sbuoy);
    return reinterpret_cast<const T *>(c->sbuoy32);
}

// FP32 copy of b' after an update from outside the stage kernels
void refresh_b32(ps3d_gpu_ctx *c)
{
    if (c->fp64 || !c->cfg.buoyancy) return;
    op_narrow(c->st, c->sbuoy, c->sbuoy32, c->d.nfield);
    c->launches += 1;
}

// semi-spectral b' into bs and the physical b' into c->buoy
// (field_combine_physical(sbuoy, buoy), inversion.f90:243)
template <typename T> void buoy_physical(ps3d_gpu_ctx *c, T *bs)
{
    col<T>(c, COL_COMBINE, sbuoy_T<T>(c), bs);
    xyi<T>(c, bs, tf<T>(c->buoy));
}

// semi-spectral z derivative of a mixed-spectral field before its
// decomposition (diffz, inversion_utils.f90:683-719): the linear part from
// the boundary rows and dphim / dphip plus the cosine transform of the
// differentiated sine series; as is scratch
template <typename T> void diffz_semi(ps3d_gpu_ctx *c, const T *fs, T *ds, T *as)
{
    const Dims &d = c->d;
    op_dz_sine<T>(d, c->st, c->rkz, fs, as);
    col<T>(c, COL_DCT, as, as);
    op_dz_join<T>(d, c->st, fs, tf<T>(c->dphim), tf<T>(c->dphip), as, ds);
    c->launches += 2;
}

// buoyancy_tendency (inversion.f90:232-292).  The reference decomposes each
// flux, differentiates it, combines it back to physical space and finally
// decomposes the sum.  D_x and D_y commute with the decomposition (the
// harmonic functions depend on |k| only, equal at a column and its partner)
// and decompose(combine(f)) = f, so the same tendency is
//   sbuoys = decompose(-D_x F(u b) - D_y F(v b) - N^2 F(w) - Dz(decompose F(w b))),
// F the forward horizontal transform, F(w) the semi-spectral w (svel) and Dz
// the semi-spectral derivative of diffz: 4 horizontal and 4 column
// transforms instead of 8 and 10.  Leaves the physical b' in c->buoy.
template <typename T> void buoyancy_tendency(ps3d_gpu_ctx *c)
{
    const Dims &d = c->d;
    const long long N = d.nfield;
    T *bs = tmpf<T>(c, 0), *fl = tmpf<T>(c, 1), *as = tmpf<T>(c, 4);
    T *fu = fl, *fv = fl + N, *fw = fl + 2 * N;
    T *sb = tf<T>(c->sbuoys);
    buoy_physical<T>(c, bs);
    op_bflux<T>(d, c->st, tf<T>(c->vel), tf<T>(c->buoy), fl);
    c->launches += 1;
    for (int k = 0; k < 3; ++k) xyf<T>(c, fl + k * N, fl + k * N);
    col<T>(c, COL_DECOMP, fw, fw);
    diffz_semi<T>(c, fw, bs, as);
    op_btend<T>(d, c->st, c->D(), fu, fv, tf<T>(c->svel) + 2 * N, bs, c->bfsq, sb);
    c->launches += 1;
    col<T>(c, COL_DECOMP, sb, sb);
}

// Maximum buoyancy frequency (advance.f90:147-168): sqrt(sqrt(max(b_x^2 +
// b_y^2 + (b_z + N^2)^2))) from the horizontal derivatives of the
// semi-spectral b' and the central z difference of the physical b'.
template <typename T> int buoyancy_frequency_max(ps3d_gpu_ctx *c, double *bfmax)
{
    const Dims &d = c->d;
    T *bs = tmpf<T>(c, 0), *bx = tmpf<T>(c, 1), *by = tmpf<T>(c, 2);
    buoy_physical<T>(c, bs);
    op_diff<T>(d, c->st, c->D(), 0, bs, bx);
    op_diff<T>(d, c->st, c->D(), 1, bs, by);
    c->launches += 2;
    xyi<T>(c, bx, bx);
    xyi<T>(c, by, by);
    op_bgrad_max<T>(d, c->st, bx, by, tf<T>(c->buoy), c->dzi, c->bfsq, c->bmax);
    c->launches += 1;
    unsigned long long bits = 0;
    cudaMemcpyAsync(&bits, c->bmax, sizeof(bits), cudaMemcpyDeviceToHost, c->st);
    const int rc = sync_check(c, "bfmax");
    if (rc) return rc;
    double mx;
    memcpy(&mx, &bits, sizeof(mx));
    *bfmax = sqrt(sqrt(mx));
    return PS3D_OK;
}

// Buoyancy diagnostics: available potential energy, buoyancy-gradient
// integral, minimum static stability, minimum Richardson number
// (field_diagnostics.f90:29-60, 351-397, 327-344, 268-287)
template <typename T> int buoyancy_diagnostics(ps3d_gpu_ctx *c, double out[4])
{
    const Dims &d = c->d;
    T *bs = tmpf<T>(c, 0), *bx = tmpf<T>(c, 1), *by = tmpf<T>(c, 2);
    buoy_physical<T>(c, bs);
    op_diff<T>(d, c->st, c->D(), 0, bs, bx);
    op_diff<T>(d, c->st, c->D(), 1, bs, by);
    c->launches += 2;
    xyi<T>(c, bx, bx);
    xyi<T>(c, by, by);
    op_bdiag<T>(d, c->st, tf<T>(c->buoy), bx, by, tf<T>(c->vor), c->dzi, c->bfsq, c->bpart, c->bres);
    c->launches += 2;
    double r[4];
    cudaMemcpyAsync(r, c->bres, sizeof(r), cudaMemcpyDeviceToHost, c->st);
    const int rc = sync_check(c, "buoyancy diagnostics");
    if (rc) return rc;
    out[0] = r[0] / (2.0 * c->bfsq) * c->ncelli;
    out[1] = r[1] * c->ncelli;
    out[2] = 1.0 + r[2] / c->bfsq;
    out[3] = r[3];
    return PS3D_OK;
}

// ------------------------------------------------------------------- source
// learned closure: the attached network's correction from the physical vor
// and vel, taken to the form svorts is assembled in (semi-spectral in the
// mixed form, mixed-spectral in FP64)
template <typename T> int closure_correction(ps3d_gpu_ctx *c)
{
    const long long N = c->d.nfield;
    T *corr = tf<T>(c->corr);
    const int rc =
        closure_apply<T>(c->closure, c->st, tf<T>(c->vor), tf<T>(c->vel), N, c->d.P, corr, N, c->closure_flags);
    c->launches += CLOSURE_LAUNCHES;
    if (rc) return check(c, "closure");
    if (sizeof(T) == sizeof(float)) {
        xyf<T>(c, corr, corr, 3);  // the three components in one launch per pass
    } else {
        for (int k = 0; k < 3; ++k) {
            xyf<T>(c, corr + k * N, corr + k * N);
            col<T>(c, COL_DECOMP, corr + k * N, corr + k * N);
        }
    }
    c->closure_fresh = false;
    return PS3D_OK;
}

template <typename T> void closure_add(ps3d_gpu_ctx *c, T *svorts)
{
    const long long N = c->d.nfield;
    for (int k = 0; k < 3; ++k) op_addf<T>(c->d, c->st, svorts + k * N, tf<T>(c->corr) + k * N);
    c->launches += 3;
}

// source (inversion.f90:376-388): buoyancy_tendency, then vorticity_tendency
// (:298-371) with the buoyancy in r = u eta - v xi + b; an attached closure's
// correction is added to the tendency
template <typename T> int source(ps3d_gpu_ctx *c)
{
    if (c->closure && ((c->closure_flags & PS3D_CLOSURE_EVERY_STAGE) || c->closure_fresh)) {
        const int rc = closure_correction<T>(c);
        if (rc) return rc;
    }
    if (c->cfg.buoyancy) buoyancy_tendency<T>(c);
    const Dims &d = c->d;
    const long long N = d.nfield;
    T *vor = tf<T>(c->vor), *vel = tf<T>(c->vel), *svorts = tf<T>(c->svorts);
    T *r = tmpf<T>(c, 0), *q = tmpf<T>(c, 1), *p = tmpf<T>(c, 2), *gq = tmpf<T>(c, 3), *gp = tmpf<T>(c, 4);
    for (int k = 0; k < 3; ++k)
        if (c->cfg.f_cor[k] != 0.0) {
            op_add_const<T>(d, c->st, vor + k * N, c->cfg.f_cor[k]);
            c->launches += 1;
        }
    // the z derivatives are taken on the physical products, as in the
    // reference: on the semi-spectral columns (where the difference commutes
    // with the horizontal transform) the FP32 form would amplify the
    // transform's rounding by 1/dz at every level, and in 256^3 and 512^3
    // runs that seeded a growing top-boundary error within about 40 steps
    T *f5[5] = {r, q, p, gq, gp};
    const bool fused_products = sizeof(T) == sizeof(float) && c->fuse_products && !c->cfg.buoyancy &&
                                lines32_prod_supported(d.ny) && r + N == q && q + N == p && p + N == gq && gq + N == gp;
    if (fused_products) {
        // the five products and their forward y lines in one launch (the
        // products stay on chip), then the x lines of each
        lines32_prod_y(c->st, reinterpret_cast<const float *>(vel), reinterpret_cast<const float *>(vor),
                       reinterpret_cast<float *>(r), d, c->dzi, tf<float2>(c->twy), &c->probe);
        c->launches += 1;
        x_forward<float>(d, c->st, reinterpret_cast<const float *>(r), reinterpret_cast<float *>(r),
                         tf<float2>(c->twx), &c->probe, 5);
        c->launches += line_launches<float>(c, d.nx, 5);
    } else if (sizeof(T) == sizeof(float)) {
        op_products_dz<float>(d, c->st, c->dzi, reinterpret_cast<const float *>(vel),
                              reinterpret_cast<const float *>(vor), tf<float>(r), tf<float>(q), tf<float>(p),
                              tf<float>(gq), tf<float>(gp));
        c->launches += 1;
    } else {
        op_products<T>(d, c->st, vel, vor, r, q, p);
        op_diffz<T>(d, c->st, c->dzi, q, gq);
        op_diffz<T>(d, c->st, c->dzi, p, gp);
        c->launches += 3;
    }
    if (c->cfg.buoyancy) {
        op_addf<T>(d, c->st, r, tf<T>(c->buoy));  // c->buoy from buoyancy_tendency
        c->launches += 1;
    }
    if (sizeof(T) == sizeof(float)) {
        // mixed: the tendency is assembled on the semi-spectral fields and
        // decomposed once per component.  The decomposition is linear per
        // column and the harmonic functions depend on |k| only, equal at a
        // column and its x / y partners, so it commutes with D_x, D_y:
        // 3 column transforms instead of 5.
        if (!fused_products) {
            if (r + N == q && q + N == p && p + N == gq && gq + N == gp) xyf<T>(c, r, r, 5);
            else
                for (int k = 0; k < 5; ++k) xyf<T>(c, f5[k], f5[k]);
        }
        if (colz_supported(d.nz)) {
            // tendency components formed inside the column kernels that
            // decompose them (the undecomposed tendency stays on chip), an
            // attached closure's correction added there
            const Deriv D = c->D();
            auto f = [](T *x) { return reinterpret_cast<float *>(x); };
            columns_src(d, c->st, f(r), f(q), f(p), f(gq), f(gp), f(svorts), f(svorts + N), f(svorts + 2 * N),
                        reinterpret_cast<float *>(c->es_src), c->k2l2, D.cx, D.cy, (float)c->dx[2],
                        (float)c->cfg.extent[2], c->twz32, c->sinz32, &c->probe,
                        c->closure ? reinterpret_cast<const float *>(c->corr) : nullptr);
            c->launches += 3;
            return check(c, "source");
        }
        op_svorts<T>(d, c->st, c->D(), r, q, p, gq, gp, svorts, svorts + N, svorts + 2 * N);
        c->launches += 1;
        if (c->closure) closure_add<T>(c, svorts);
        source_decompose_mixed<T>(c);
        return check(c, "source");
    }
    for (int k = 0; k < 5; ++k) {
        xyf<T>(c, f5[k], f5[k]);
        col<T>(c, COL_DECOMP, f5[k], f5[k]);
    }
    op_svorts<T>(d, c->st, c->D(), r, q, p, gq, gp, svorts, svorts + N, svorts + 2 * N);
    c->launches += 1;
    if (c->closure) closure_add<T>(c, svorts);
    return check(c, "source");
}

// -------------------------------------------------------------- diagnostics
template <typename T> int energy(ps3d_gpu_ctx *c, double out[RED1_N])
{
    red_pass1<T>(c->d, c->st, tf<T>(c->vel), tf<T>(c->vor), c->part, c->res1);
    c->launches += 2;
    cudaMemcpyAsync(out, c->res1, RED1_N * sizeof(double), cudaMemcpyDeviceToHost, c->st);
    return sync_check(c, "energy");
}

int set_diffusion(ps3d_gpu_ctx *c, double dt, double pref, double bpref);

// get_diffusion_pre_factor (advance.f90:381-410)
double pre_factor(int pretype, double vorch, double bfmax, double rmv, double rmb, double ggmax, double usggmax)
{
    switch (pretype) {
    case PS3D_PRE_CONSTANT: return 1.0;
    case PS3D_PRE_VORCH: return vorch;
    case PS3D_PRE_BFMAX: return bfmax;
    case PS3D_PRE_ROLL_MEAN_BFMAX: return rmb;
    case PS3D_PRE_MAX_STRAIN: return ggmax;
    case PS3D_PRE_US_MAX_STRAIN: return usggmax;
    default: return rmv;
    }
}

// adapt (advance.f90:109-377)
// internal: the state advance_host received differs from the device's;
// the staged state has been installed and projected, and the first
// right-hand side must be evaluated again (never leaves the library)
constexpr int RESTART_STATE = -1000;

// Wait for advance_host's state check.  Unchanged: nothing to do (the step
// runs on the device state, bitwise the host's).  Changed: the staged host
// state becomes the state, projected in FP64 as set_field does, and the
// caller starts the step over.
int resolve_state_check(ps3d_gpu_ctx *c)
{
    c->pending_check = false;
    int changed = 0;
    cudaStreamWaitEvent(c->st, c->ev_chk, 0);
    cudaMemcpyAsync(&changed, c->flag_chk, sizeof(int), cudaMemcpyDeviceToHost, c->st);
    int rc = sync_check(c, "advance_host");
    if (rc) return rc;
    if (!changed) return PS3D_OK;
    // levels 0..nz of every column (the staging array's padding rows hold
    // whatever the accumulator left there)
    const size_t pitch = (size_t)c->d.P * sizeof(double);
    cudaMemcpy2DAsync(c->svor, pitch, c->svorf, pitch, (size_t)(c->d.nz + 1) * sizeof(double), (size_t)3 * c->d.ncol,
                      cudaMemcpyDeviceToDevice, c->st);
    project_state_mixed(c);
    rc = check(c, "advance_host");
    return rc ? rc : RESTART_STATE;
}

template <typename T> int adapt(ps3d_gpu_ctx *c, double t, double *dt_out, ps3d_gpu_diag *diag)
{
    const Dims &d = c->d;
    double bfmax = 0.0;
    int rc;
    if (c->cfg.buoyancy) {
        rc = buoyancy_frequency_max<T>(c, &bfmax);
        if (rc) return rc;
    }
    double r1[RED1_N];
    rc = energy<T>(c, r1);
    if (rc) return rc;
    const double vortmax = sqrt(r1[0]);
    const double vortrms = sqrt(r1[1] / (double)c->ncell);
    // velocity gradients (5 inverse transforms)
    T *g5 = tmpf<T>(c, 0);
    op_strain_fields<T>(d, c->st, c->D(), tf<T>(c->svel), g5);
    c->launches += 1;
    xyi<T>(c, g5, g5, 5);
    cudaMemsetAsync(c->flag, 0, sizeof(int), c->st);
    red_pass2<T>(d, c->st, tf<T>(c->vor), g5, vortrms, c->part, c->res2, c->flag);
    c->launches += 2;
    double r2[RED2_N];
    int hflag = 0;
    cudaMemcpyAsync(r2, c->res2, RED2_N * sizeof(double), cudaMemcpyDeviceToHost, c->st);
    cudaMemcpyAsync(&hflag, c->flag, sizeof(int), cudaMemcpyDeviceToHost, c->st);
    rc = sync_check(c, "adapt");
    if (rc) return rc;
    if (hflag) return fail(c, PS3D_ERR_DEVICE_LIMIT, "adapt: Jacobi sweep limit reached");
    if (lines32_error()) return fail(c, PS3D_ERR_DEVICE_LIMIT, "line transform: a wait for a tile copy ran out");
    if (colz_error()) return fail(c, PS3D_ERR_DEVICE_LIMIT, "column transform: a staged copy wait ran out or a layout was refused");
    const double small = 1.0e-12;
    const double vorch = r2[1] / (small + r2[0]);
    const double ggmax = r2[2], usggmax = r2[3], lsggmax = r2[4];
    const double umax = r1[7], vmax = r1[8], wmax = r1[9];
    const double dtcfl = c->cfg.cflmax * fmin(fmin(c->dx[0] / (umax + small), c->dx[1] / (vmax + small)),
                                              c->dx[2] / (wmax + small));
    const double dt = fmin(fmin(c->cfg.alpha / (ggmax + small), c->cfg.alpha / (bfmax + small)),
                           fmin(dtcfl, c->cfg.time_limit - t));
    // the buoyancy rolling mean is taken before the strain one (:358-366)
    const double rmb = c->cfg.buoyancy ? c->roll_b.next(bfmax) : 0.0;
    const double rmv = c->roll.next(ggmax);
    const double val = pre_factor(c->cfg.pretype, vorch, bfmax, rmv, rmb, ggmax, usggmax);
    const double bval =
        c->cfg.buoyancy ? pre_factor(c->cfg.buoy_pretype, vorch, bfmax, rmv, rmb, ggmax, usggmax) : 0.0;
    if (!std::isfinite(dt) || !std::isfinite(r1[1]) || !std::isfinite(r1[2]) || !std::isfinite(bfmax))
        return fail(c, PS3D_ERR_NONFINITE, "adapt: non-finite diagnostic");
    rc = set_diffusion(c, dt, val, bval);
    if (rc) return rc;
    if (diag) {
        diag->t = t;
        diag->dt = dt;
        diag->ke = 0.5 * r1[2] * c->ncelli;
        diag->en = 0.5 * r1[1] * c->ncelli;
        diag->hel = r1[3] * c->ncelli;
        diag->vortmax = vortmax;
        diag->vortrms = vortrms;
        diag->vorch = vorch;
        for (int k = 0; k < 3; ++k) diag->vormean[k] = r1[4 + k] * c->ncelli;
        diag->ggmax = ggmax;
        diag->usggmax = usggmax;
        diag->lsggmax = lsggmax;
        diag->umax = umax;
        diag->vmax = vmax;
        diag->wmax = wmax;
        diag->bfmax = bfmax;
        diag->rmv = rmv;
        diag->pref = val;
        diag->rmb = rmb;
        diag->bpref = bval;
    }
    *dt_out = dt;
    return PS3D_OK;
}

// ----------------------------------------------------------------- steppers
__global__ void k_vdiss(long long n, const double *vhdis, double *vdiss, double dfac, int cn2)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vdiss[i] = cn2 ? 1.0 / (1.0 + dfac * vhdis[i]) : dfac * vhdis[i];
}

int set_diffusion(ps3d_gpu_ctx *c, double dt, double pref, double bpref)
{
    if (!c->diffusion_ready) return fail(c, PS3D_ERR_NOT_READY, "set_diffusion before init_diffusion");
    const bool cn2 = c->cfg.stepper == PS3D_CN2;
    const unsigned nb = (unsigned)((c->d.ncol + 255) / 256);
    // impl_rk4_set_diffusion (impl_rk4.f90:37-53), cn2_set_diffusion (cn2.f90:40-77)
    const double dfac = cn2 ? ((c->cfg.nnu == 1) ? dt : pref * dt) : 0.5 * pref * dt;
    k_vdiss<<<nb, 256, 0, c->st>>>(c->d.ncol, c->vhdis, c->vdiss, dfac, cn2);
    c->launches += 1;
    if (c->cfg.buoyancy) {
        const double dbac = cn2 ? ((c->cfg.buoy_nnu == 1) ? dt : bpref * dt) : 0.5 * bpref * dt;
        k_vdiss<<<nb, 256, 0, c->st>>>(c->d.ncol, c->bhdis, c->bdiss, dbac, cn2);
        c->launches += 1;
    }
    return check(c, "set_diffusion");
}

template <typename T> int rhs_or_hold(ps3d_gpu_ctx *c)
{
    if (c->cfg.hold_source) {
        cudaMemcpyAsync(c->svorts, c->held, 3 * c->d.nfield * sizeof(T), cudaMemcpyDeviceToDevice, c->st);
        if (!c->fp64)
            cudaMemcpyAsync(c->es_src, tf<T>(c->held) + 3 * c->d.nfield, c->d.nfield * sizeof(T),
                            cudaMemcpyDeviceToDevice, c->st);
        if (c->cfg.buoyancy)
            cudaMemcpyAsync(c->sbuoys, c->heldb, c->d.nfield * sizeof(T), cudaMemcpyDeviceToDevice, c->st);
        return check(c, "hold");
    }
    int rc = vor2vel<T>(c);
    if (rc) return rc;
    return source<T>(c);
}

// impl_rk4_step (impl_rk4.f90:76-207)
__global__ void k_set_dt(StepScal *sc, double dt) { sc->dt = dt; }

// column factors of impl-diff-rk4 substep sub (impl_rk4.f90:212-364):
// the multiplier of the source (fp) and the integrating factor (fm)
void stage_factors(ps3d_gpu_ctx *c, int sub, const double **fp, const double **fm)
{
    switch (sub) {
    case 1: *fp = c->filt0; *fm = c->emq; break;
    case 2: *fp = c->epq; *fm = c->emq; break;
    case 3: *fp = c->epq; *fm = c->emq2; break;
    default: *fp = c->epq2; *fm = c->emq2; break;
    }
}

// the mixed form's fused projection, filter and stage update of substep sub
void stage_mixed(ps3d_gpu_ctx *c, int sub)
{
    const double *fp, *fm;
    stage_factors(c, sub, &fp, &fm);
    op_stage_orbit(c->d, c->st, sub, c->D(), c->k2l2i, tf<float>(c->svorts), c->es_src, c->svor,
                   reinterpret_cast<float *>(c->svorf), c->svor32, c->mf64, fp, fm, &c->sc->dt);
    c->launches += 1;
}

// t == nullptr: a device-driven step (dt already in c->sc, the time kept on
// the device); only the mixed form runs that way
template <typename T> int step_rk4(ps3d_gpu_ctx *c, double *t, double dt)
{
    const Dims &d = c->d;
    const long long N = d.nfield;
    const double dt2 = 0.5 * dt, dt3 = dt / 3.0, dt6 = dt / 6.0;
    T *sv = tf<T>(c->svorts);
    const double *dtp = &c->sc->dt;
    if (sizeof(T) == sizeof(float) && t) {
        k_set_dt<<<1, 1, 0, c->st>>>(c->sc, dt);
        c->launches += 1;
    }
    const bool buoy = c->cfg.buoyancy != 0;
    if (c->cfg.hold_source) {
        cudaMemcpyAsync(c->held, c->svorts, 3 * N * sizeof(T), cudaMemcpyDeviceToDevice, c->st);
        if (!c->fp64)
            cudaMemcpyAsync(tf<T>(c->held) + 3 * N, c->es_src, N * sizeof(T), cudaMemcpyDeviceToDevice, c->st);
        if (buoy) cudaMemcpyAsync(c->heldb, c->sbuoys, N * sizeof(T), cudaMemcpyDeviceToDevice, c->st);
    }
    op_rk4_factors(d, c->st, c->vdiss, c->filt0, c->epq, c->emq, c->epq2, c->emq2);
    c->launches += 1;
    if (buoy) {
        op_rk4_factors(d, c->st, c->bdiss, c->filt0, c->bpq, c->bmq, c->bpq2, c->bmq2);
        c->launches += 1;
    }
    const bool mixed = sizeof(T) == sizeof(float);
    float *s32 = reinterpret_cast<float *>(sv), *q32 = c->svor32;
    // mixed: the accumulator's FP32 increments live in the (FP64-sized) svorf
    float *acc = reinterpret_cast<float *>(c->svorf);
    // buoyancy: the same substeps with its own factors (impl_rk4.f90:99-195)
    T *sb = tf<T>(c->sbuoys);
    float *sb32 = reinterpret_cast<float *>(sb), *accb = reinterpret_cast<float *>(c->sbuoyf);
    if (buoy) {
        if (mixed)
            op_rk4m_sub1(d, c->st, c->sbuoy, c->sbuoyi, accb, sb32, c->sbuoy32, c->filt0, c->bmq, dtp);
        else
            op_rk4_sub1<T>(d, c->st, c->sbuoy, c->sbuoyi, c->sbuoyf, sb, c->filt0, c->bmq, dt2, dt6);
        c->launches += 1;
    }
    // the mixed form: projection, filter and stage update in one pass per
    // substep (op_stage_orbit); the FP64 state keeps the step's initial
    // state until substep 4, and vor2vel reads the stage state's (0,0)
    // column from mf64 meanwhile
    struct MeanFlowSource {
        ps3d_gpu_ctx *c;
        ~MeanFlowSource() { c->mf_a = nullptr; }
    } mf_guard{c};
    auto stage = [&](int sub, const double *, const double *) {
        stage_mixed(c, sub);
        c->mf_a = sub < 4 ? c->mf64 : nullptr;
    };
    if (mixed) {
        stage(1, c->filt0, c->emq);
    } else {
        for (int k = 0; k < 3; ++k)
            op_rk4_sub1<T>(d, c->st, c->svor + k * N, c->svori + k * N, c->svorf + k * N, sv + k * N, c->filt0,
                           c->emq, dt2, dt6);
        c->launches += 3;
    }
    int rc = rhs_or_hold<T>(c);
    if (rc) return rc;
    if (t) *t += dt2;
    if (buoy) {
        if (mixed)
            op_rk4m_sub23(d, c->st, c->sbuoy, c->sbuoyi, accb, sb32, c->sbuoy32, c->bpq, c->bmq, dtp, false);
        else
            op_rk4_sub23<T>(d, c->st, c->sbuoy, c->sbuoyi, c->sbuoyf, sb, c->bpq, c->bmq, dt2, dt3);
        c->launches += 1;
    }
    if (mixed) {
        stage(2, c->epq, c->emq);
    } else {
        for (int k = 0; k < 3; ++k)
            op_rk4_sub23<T>(d, c->st, c->svor + k * N, c->svori + k * N, c->svorf + k * N, sv + k * N, c->epq,
                            c->emq, dt2, dt3);
        c->launches += 3;
    }
    rc = rhs_or_hold<T>(c);
    if (rc) return rc;
    if (t) *t += dt2;
    if (buoy) {
        if (mixed)
            op_rk4m_sub23(d, c->st, c->sbuoy, c->sbuoyi, accb, sb32, c->sbuoy32, c->bpq, c->bmq2, dtp, true);
        else
            op_rk4_sub23<T>(d, c->st, c->sbuoy, c->sbuoyi, c->sbuoyf, sb, c->bpq, c->bmq2, dt, dt3);
        c->launches += 1;
    }
    if (mixed) {
        stage(3, c->epq, c->emq2);
    } else {
        for (int k = 0; k < 3; ++k)
            op_rk4_sub23<T>(d, c->st, c->svor + k * N, c->svori + k * N, c->svorf + k * N, sv + k * N, c->epq,
                            c->emq2, dt, dt3);
        c->launches += 3;
    }
    rc = rhs_or_hold<T>(c);
    if (rc) return rc;
    if (buoy) {
        if (mixed)
            op_rk4m_sub4(d, c->st, c->sbuoy, c->sbuoyi, accb, sb32, c->sbuoy32, c->bpq2, c->bmq2, dtp);
        else
            op_rk4_sub4<T>(d, c->st, c->sbuoy, c->sbuoyf, sb, c->bpq2, c->bmq2, dt6);
        c->launches += 1;
    }
    if (mixed) {
        stage(4, c->epq2, c->emq2);
    } else {
        for (int k = 0; k < 3; ++k)
            op_rk4_sub4<T>(d, c->st, c->svor + k * N, c->svorf + k * N, sv + k * N, c->epq2, c->emq2, dt6);
        c->launches += 3;
    }
    op_mean_fix(d, c->st, c->svor, c->dstsum, c->fnzi, c->ini, nullptr, 1, c->svor32);
    c->launches += 1;
    return check(c, "step");
}

// cn2_step (cn2.f90:92-181)
template <typename T> int step_cn2(ps3d_gpu_ctx *c, double *t, double dt)
{
    const Dims &d = c->d;
    const double dt2 = 0.5 * dt;
    T *sv = tf<T>(c->svorts), *sb = tf<T>(c->sbuoys);
    const bool buoy = c->cfg.buoyancy != 0;
    if (c->cfg.hold_source) {
        cudaMemcpyAsync(c->held, c->svorts, 3 * d.nfield * sizeof(T), cudaMemcpyDeviceToDevice, c->st);
        if (buoy) cudaMemcpyAsync(c->heldb, c->sbuoys, d.nfield * sizeof(T), cudaMemcpyDeviceToDevice, c->st);
    }
    // the mixed form re-projects in FP64 after each update: the 3-D filter of
    // cn2 does not commute with the projection
    const bool mixed = sizeof(T) == sizeof(float);
    // buoyancy first (cn2.f90:107-117, 151-160)
    if (buoy) {
        op_cn2_init<T>(d, c->st, c->bsm, c->sbuoy, sb, dt2, 1);
        op_cn2_update<T>(d, c->st, c->sbuoy, c->bsm, sb, c->filt0, c->fz, c->bdiss, dt2, 1);
        refresh_b32(c);
        c->launches += 2;
    }
    op_cn2_init<T>(d, c->st, c->vortsm, c->svor, sv, dt2);
    op_cn2_update<T>(d, c->st, c->svor, c->vortsm, sv, c->filt0, c->fz, c->vdiss, dt2);
    op_mean_fix(d, c->st, c->svor, c->dstsum, c->fnzi, c->ini, nullptr, 1);
    if (mixed) project_state_mixed(c);
    c->launches += 7;
    for (int it = 0; it < 2; ++it) {
        int rc = rhs_or_hold<T>(c);
        if (rc) return rc;
        if (buoy) {
            op_cn2_update<T>(d, c->st, c->sbuoy, c->bsm, sb, c->filt0, c->fz, c->bdiss, dt2, 1);
            refresh_b32(c);
            c->launches += 1;
        }
        op_cn2_update<T>(d, c->st, c->svor, c->vortsm, sv, c->filt0, c->fz, c->vdiss, dt2);
        op_mean_fix(d, c->st, c->svor, c->dstsum, c->fnzi, c->ini, nullptr, 1);
        if (mixed) project_state_mixed(c);
        c->launches += 4;
    }
    *t += dt;
    return check(c, "step");
}

template <typename T> int step(ps3d_gpu_ctx *c, double *t, double dt)
{
    if (!c->diffusion_ready) return fail(c, PS3D_ERR_NOT_READY, "step before init_diffusion");
    return c->cfg.stepper == PS3D_CN2 ? step_cn2<T>(c, t, dt) : step_rk4<T>(c, t, dt);
}

// advance (advance.f90:77-104)
template <typename T> int advance(ps3d_gpu_ctx *c, double *t, ps3d_gpu_diag *diag)
{
    // advance_host's state check runs beside the first right-hand side
    // (vor2vel, adapt, source), which writes transient fields and, on the
    // host, adapt's rolling means (kept here to be put back) and the
    // diffusion tables (rebuilt by a second adapt); it is resolved before the
    // stage updates touch the state
    Rolling keep_roll, keep_roll_b;
    if (c->pending_check) {
        keep_roll = c->roll;
        keep_roll_b = c->roll_b;
    }
    double dt = 0.0;
    for (int pass = 0; pass < 2; ++pass) {
        int rc = vor2vel<T>(c);
        if (rc) return rc;
        rc = adapt<T>(c, *t, &dt, diag);
        if (rc) return rc;
        c->closure_fresh = true;
        rc = source<T>(c);
        if (rc) return rc;
        if (!c->pending_check) break;
        rc = resolve_state_check(c);
        if (rc != RESTART_STATE) {
            if (rc) return rc;
            break;
        }
        // the host state differed: it is installed and projected; evaluate
        // the right-hand side again from it
        c->roll = keep_roll;
        c->roll_b = keep_roll_b;
    }
    return step<T>(c, t, dt);
}

// ------------------------------------------------- device-driven step
// adapt's scalar logic (advance.f90:109-377, rolling_mean.f90:36-69) on the
// device, one thread, the same operations in the same order as the host
// version in adapt<T>; results stay in c->sc for the stage kernels.
struct AdaptParams {
    double cflmax, alpha, time_limit, dx0, dx1, dx2, ncell, ncelli;
    int pretype, L;
};

__global__ void k_adapt_scalars(StepScal *sc, double *hist, const double *__restrict__ r1,
                                const double *__restrict__ r2, const int *__restrict__ flag, AdaptParams p)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double t = sc->t;
    const double small = 1.0e-12;
    const double vortmax = sqrt(r1[0]);
    const double vortrms = sqrt(r1[1] / p.ncell);
    const double vorch = r2[1] / (small + r2[0]);
    const double ggmax = r2[2], usggmax = r2[3], lsggmax = r2[4];
    const double umax = r1[7], vmax = r1[8], wmax = r1[9];
    const double bfmax = 0.0;
    const double dtcfl =
        p.cflmax * fmin(fmin(p.dx0 / (umax + small), p.dx1 / (vmax + small)), p.dx2 / (wmax + small));
    const double dt = fmin(fmin(p.alpha / (ggmax + small), p.alpha / (bfmax + small)), fmin(dtcfl, p.time_limit - t));
    double sma;
    const int L = p.L;
    if (sc->filled) {
        const double vold = hist[sc->iold - 1];
        sc->iold = sc->iold % L + 1;
        sma = sc->sma + (ggmax - vold) / (double)L;
        hist[sc->inew - 1] = ggmax;
        sc->inew = sc->inew % L + 1;
    } else {
        hist[sc->inew - 1] = ggmax;
        double sum = 0.0;
        for (int i = 0; i < sc->inew; ++i) sum += hist[i];
        sma = sum / (double)sc->inew;
        sc->filled = (L == sc->inew);
        sc->inew = sc->inew % L + 1;
    }
    sc->sma = sma;
    double val;
    switch (p.pretype) {
    case PS3D_PRE_CONSTANT: val = 1.0; break;
    case PS3D_PRE_VORCH: val = vorch; break;
    case PS3D_PRE_BFMAX: val = bfmax; break;
    case PS3D_PRE_MAX_STRAIN: val = ggmax; break;
    case PS3D_PRE_US_MAX_STRAIN: val = usggmax; break;
    default: val = sma; break;
    }
    if (*flag) sc->err |= 2;
    if (!isfinite(dt) || !isfinite(r1[1]) || !isfinite(r1[2])) sc->err |= 1;
    sc->dt = dt;
    sc->dfac = 0.5 * val * dt;  // impl_rk4_set_diffusion (impl_rk4.f90:37-53)
    double *g = sc->diag;
    g[0] = t;
    g[1] = dt;
    g[2] = 0.5 * r1[2] * p.ncelli;
    g[3] = 0.5 * r1[1] * p.ncelli;
    g[4] = r1[3] * p.ncelli;
    g[5] = vortmax;
    g[6] = vortrms;
    g[7] = vorch;
    for (int k = 0; k < 3; ++k) g[8 + k] = r1[4 + k] * p.ncelli;
    g[11] = ggmax;
    g[12] = usggmax;
    g[13] = lsggmax;
    g[14] = umax;
    g[15] = vmax;
    g[16] = wmax;
    g[17] = bfmax;
    g[18] = sma;
    g[19] = val;
    g[20] = 0.0;  // no buoyancy in captured steps
    g[21] = 0.0;
    // the stepper advances t by dt/2 twice (impl_rk4.f90)
    const double dt2 = 0.5 * dt;
    sc->t = (t + dt2) + dt2;
}

__global__ void k_vdiss_dev(long long n, const double *vhdis, double *vdiss, const StepScal *sc)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vdiss[i] = sc->dfac * vhdis[i];
}

// One advance of the mixed form with impl-diff-rk4 and no host
// synchronisation, in the pieces a batch interleaves with the stage updates
// of its other runs: dev_pre (vor2vel, adapt on the device, the first
// source and the integrating factors), then for substeps 1..4 the stage
// update, with dev_rhs (vor2vel and source of the stage state) between
// them, and dev_end (the vorticity-mean fix).  The same kernels in the same
// order as advance<float> with step_rk4<float>.
int dev_pre(ps3d_gpu_ctx *c)
{
    const Dims &d = c->d;
    const long long N = d.nfield;
    int rc = vor2vel<float>(c);
    if (rc) return rc;
    red_pass1<float>(d, c->st, tf<float>(c->vel), tf<float>(c->vor), c->part, c->res1);
    float *g5 = tmpf<float>(c, 0);
    op_strain_fields<float>(d, c->st, c->D(), tf<float>(c->svel), g5);
    c->launches += 3;
    for (int k = 0; k < 5; ++k) xyi<float>(c, g5 + k * N, g5 + k * N);
    cudaMemsetAsync(c->flag, 0, sizeof(int), c->st);
    red_pass2<float>(d, c->st, tf<float>(c->vor), g5, 0.0, c->part, c->res2, c->flag, c->res1, (double)c->ncell);
    c->launches += 2;
    AdaptParams ap;
    ap.cflmax = c->cfg.cflmax;
    ap.alpha = c->cfg.alpha;
    ap.time_limit = c->cfg.time_limit;
    ap.dx0 = c->dx[0];
    ap.dx1 = c->dx[1];
    ap.dx2 = c->dx[2];
    ap.ncell = (double)c->ncell;
    ap.ncelli = c->ncelli;
    ap.pretype = c->cfg.pretype;
    ap.L = (int)c->roll.hist.size();
    k_adapt_scalars<<<1, 1, 0, c->st>>>(c->sc, c->roll_dev, c->res1, c->res2, c->flag, ap);
    k_vdiss_dev<<<(unsigned)((d.ncol + 255) / 256), 256, 0, c->st>>>(d.ncol, c->vhdis, c->vdiss, c->sc);
    c->launches += 2;
    c->closure_fresh = true;
    rc = source<float>(c);
    if (rc) return rc;
    op_rk4_factors(d, c->st, c->vdiss, c->filt0, c->epq, c->emq, c->epq2, c->emq2);
    c->launches += 1;
    return check(c, "advance");
}

int dev_rhs(ps3d_gpu_ctx *c)
{
    c->mf_a = c->mf64;
    int rc = vor2vel<float>(c);
    if (!rc) rc = source<float>(c);
    c->mf_a = nullptr;
    return rc;
}

void dev_end(ps3d_gpu_ctx *c)
{
    op_mean_fix(c->d, c->st, c->svor, c->dstsum, c->fnzi, c->ini, nullptr, 1, c->svor32);
    c->launches += 1;
}

int advance_dev(ps3d_gpu_ctx *c)
{
    int rc = dev_pre(c);
    for (int sub = 1; sub <= 4 && !rc; ++sub) {
        stage_mixed(c, sub);
        if (sub < 4) rc = dev_rhs(c);
    }
    if (rc) return rc;
    dev_end(c);
    return check(c, "advance");
}

int graph_supported(ps3d_gpu_ctx *c)
{
    if (c->fp64 || c->cfg.stepper == PS3D_CN2 || c->cfg.hold_source || c->cfg.buoyancy)
        return fail(c, PS3D_ERR_INVALID_ARG,
                    "captured steps need the mixed form, impl-diff-rk4, no held source, no buoyancy");
    if (!c->diffusion_ready) return fail(c, PS3D_ERR_NOT_READY, "advance before init_diffusion");
    return PS3D_OK;
}

// upload the model time and the rolling-mean state for device-driven steps
int graph_upload(ps3d_gpu_ctx *c, double t)
{
    int rc = graph_supported(c);
    if (rc) return rc;
    StepScal h{};
    h.t = t;
    h.sma = c->roll.sma;
    h.inew = c->roll.inew;
    h.iold = c->roll.iold;
    h.filled = c->roll.filled ? 1 : 0;
    cudaMemcpyAsync(c->sc, &h, sizeof(h), cudaMemcpyHostToDevice, c->st);
    cudaMemcpyAsync(c->roll_dev, c->roll.hist.data(), c->roll.hist.size() * sizeof(double),
                    cudaMemcpyHostToDevice, c->st);
    return sync_check(c, "graph_prepare");
}

// upload the scalars; capture the step once
int graph_prepare(ps3d_gpu_ctx *c, double t)
{
    int rc = graph_upload(c, t);
    if (rc) return rc;
    if (c->graph) return PS3D_OK;
    const int kind = c->probe.kind;
    c->probe.kind = PROBE_OFF;  // no event records inside the graph
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        c->probe.kind = kind;
        return check(c, "graph capture");
    }
    const long long l0 = c->launches;
    rc = advance_dev(c);
    const cudaError_t e = cudaStreamEndCapture(c->st, &g);
    c->probe.kind = kind;
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc ? rc : fail(c, PS3D_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    }
    c->graph_launches = c->launches - l0;
    c->launches = l0;
    const cudaError_t ei = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        c->graph = nullptr;
        return fail(c, PS3D_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
    }
    return PS3D_OK;
}

int graph_launch(ps3d_gpu_ctx *c, int nsteps)
{
    for (int s = 0; s < nsteps; ++s)
        if (cudaGraphLaunch(c->graph, c->st) != cudaSuccess) return check(c, "graph launch");
    c->launches += c->graph_launches * nsteps;
    return PS3D_OK;
}

// read back the time, the last step's diagnostics and the rolling state
int graph_finish(ps3d_gpu_ctx *c, double *t, ps3d_gpu_diag *diag)
{
    StepScal h;
    cudaMemcpyAsync(&h, c->sc, sizeof(h), cudaMemcpyDeviceToHost, c->st);
    cudaMemcpyAsync(c->roll.hist.data(), c->roll_dev, c->roll.hist.size() * sizeof(double),
                    cudaMemcpyDeviceToHost, c->st);
    int rc = sync_check(c, "graph_finish");
    if (rc) return rc;
    if (lines32_error()) return fail(c, PS3D_ERR_DEVICE_LIMIT, "line transform: a wait for a tile copy ran out");
    if (colz_error()) return fail(c, PS3D_ERR_DEVICE_LIMIT, "column transform: a staged copy wait ran out or a layout was refused");
    c->roll.sma = h.sma;
    c->roll.inew = h.inew;
    c->roll.iold = h.iold;
    c->roll.filled = h.filled != 0;
    *t = h.t;
    if (diag) {
        static_assert(sizeof(ps3d_gpu_diag) == 22 * sizeof(double), "diag layout");
        memcpy(diag, h.diag, sizeof(h.diag));
    }
    if (h.err & 2) return fail(c, PS3D_ERR_DEVICE_LIMIT, "adapt: Jacobi sweep limit reached");
    if (h.err & 1) return fail(c, PS3D_ERR_NONFINITE, "adapt: non-finite diagnostic");
    return PS3D_OK;
}

// ------------------------------------------------------------ batch step
// A batch of independent runs (any grid sizes, mixed form, impl-diff-rk4)
// advanced one whole step per CUDA graph launch: every run's pieces of the
// device-driven advance run on the run's own stream, and each of the four
// stage updates is one persistent launch over the (run, partner orbit) work
// items of all runs (op_batch_stage), between a join of all runs' streams
// and a fork back to them.
struct BatchPlan {
    std::vector<ps3d_gpu_ctx *> runs;
    std::vector<unsigned long long> serials;
    std::vector<cudaEvent_t> ev;  // fork (0) and one join event per run
    cudaGraphExec_t exec = nullptr;
    StageRun *dev_runs = nullptr;
    long long nitems = 0, kernels = 0;
    int blocks = 0;
    ~BatchPlan()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (dev_runs) cudaFree(dev_runs);
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
    bool same(ps3d_gpu_ctx *const *ctx, int n) const
    {
        if ((int)runs.size() != n) return false;
        for (int i = 0; i < n; ++i)
            if (runs[i] != ctx[i] || serials[i] != ctx[i]->serial) return false;
        return true;
    }
};

int batch_capture(BatchPlan *bp)
{
    const int n = (int)bp->runs.size();
    ps3d_gpu_ctx *c0 = bp->runs[0];
    cudaStream_t s0 = c0->st;
    std::vector<StageRun> h(n);
    long long items = 0;
    for (int i = 0; i < n; ++i) {
        ps3d_gpu_ctx *c = bp->runs[i];
        StageRun &r = h[i];
        r.d = c->d;
        r.D = c->D();
        r.k2l2i = c->k2l2i;
        r.S = tf<float>(c->svorts);
        r.es = c->es_src;
        r.q = c->svor;
        r.acc = reinterpret_cast<float *>(c->svorf);
        r.q32 = c->svor32;
        r.mf = c->mf64;
        for (int sub = 1; sub <= 4; ++sub) stage_factors(c, sub, &r.fp[sub - 1], &r.fm[sub - 1]);
        r.dtp = &c->sc->dt;
        r.item0 = items;
        items += (long long)(c->d.nx / 2 + 1) * (c->d.ny / 2 + 1);
    }
    bp->nitems = items;
    bp->blocks = batch_stage_blocks();
    if (cudaMalloc(&bp->dev_runs, n * sizeof(StageRun)) != cudaSuccess) {
        cudaGetLastError();
        return fail(c0, PS3D_ERR_OUT_OF_MEMORY, "batch: run table");
    }
    cudaMemcpyAsync(bp->dev_runs, h.data(), n * sizeof(StageRun), cudaMemcpyHostToDevice, s0);
    bp->ev.assign(n + 1, nullptr);
    for (auto &e : bp->ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    int rc = sync_check(c0, "batch set-up");
    if (rc) return rc;
    std::vector<int> kinds(n);
    for (int i = 0; i < n; ++i) {
        kinds[i] = bp->runs[i]->probe.kind;
        bp->runs[i]->probe.kind = PROBE_OFF;  // no event records inside the graph
    }
    std::vector<long long> l0(n);
    for (int i = 0; i < n; ++i) l0[i] = bp->runs[i]->launches;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = check(c0, "batch capture");
    auto fork = [&]() {
        cudaEventRecord(bp->ev[0], s0);
        for (int i = 1; i < n; ++i) cudaStreamWaitEvent(bp->runs[i]->st, bp->ev[0], 0);
    };
    auto join = [&]() {
        for (int i = 1; i < n; ++i) {
            cudaEventRecord(bp->ev[i], bp->runs[i]->st);
            cudaStreamWaitEvent(s0, bp->ev[i], 0);
        }
    };
    long long stage_launches = 0;
    if (!rc) {
        fork();
        for (int i = 0; i < n && !rc; ++i) rc = dev_pre(bp->runs[i]);
        join();
        for (int sub = 1; sub <= 4 && !rc; ++sub) {
            op_batch_stage(s0, sub, bp->dev_runs, n, bp->nitems, bp->blocks);
            ++stage_launches;
            if (sub < 4) {
                fork();
                for (int i = 0; i < n && !rc; ++i) rc = dev_rhs(bp->runs[i]);
                join();
            }
        }
        if (!rc) {
            fork();
            for (int i = 0; i < n; ++i) dev_end(bp->runs[i]);
            join();
        }
        const cudaError_t e = cudaStreamEndCapture(s0, &g);
        if (!rc && e != cudaSuccess) rc = fail(c0, PS3D_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
    }
    long long kernels = stage_launches;
    for (int i = 0; i < n; ++i) {
        bp->runs[i]->probe.kind = kinds[i];
        kernels += bp->runs[i]->launches - l0[i];
        bp->runs[i]->launches = l0[i];
    }
    bp->kernels = kernels;
    if (rc) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc;
    }
    const cudaError_t ei = cudaGraphInstantiate(&bp->exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        bp->exec = nullptr;
        return fail(c0, PS3D_ERR_CUDA, std::string("batch instantiate: ") + cudaGetErrorString(ei));
    }
    return PS3D_OK;
}

// ---------------------------------------------------------- derived fields
// pressure and horizontal divergence (fields_derived.f90:67-182) from the
// current vel / vor / svel (and b' on buoyancy contexts); physical fields to
// the host
template <typename T> int derived_fields(ps3d_gpu_ctx *c, double *hp, double *hd)
{
    const Dims &d = c->d;
    const long long N = d.nfield;
    if (hp) {
        T *g5 = tmpf<T>(c, 0), *pr = tmpf<T>(c, 5);
        op_strain_fields<T>(d, c->st, c->D(), tf<T>(c->svel), g5);
        c->launches += 1;
        for (int k = 0; k < 5; ++k) xyi<T>(c, g5 + k * N, g5 + k * N);
        op_pressure_rhs<T>(d, c->st, g5, tf<T>(c->vor), pr);
        c->launches += 1;
        if (c->cfg.buoyancy) {
            buoy_physical<T>(c, g5);
            op_pres_buoy_rhs<T>(d, c->st, tf<T>(c->buoy), tf<T>(c->vor) + 2 * N, c->dzi, c->cfg.f_cor[2], pr);
            c->launches += 1;
        }
        xyf<T>(c, pr, pr);
        col<T>(c, COL_DCT, pr, pr);
        op_mul_field<T>(d, c->st, tf<T>(c->green), pr);
        c->launches += 1;
        col<T>(c, COL_DCT, pr, pr);
        if (c->cfg.buoyancy) {
            op_pres_buoy_bc<T>(d, c->st, sbuoy_T<T>(c), c->k2l2i, tf<T>(c->dphim), tf<T>(c->dphip), pr);
            c->launches += 1;
        }
        xyi<T>(c, pr, pr);
        int rc = download(c, pr, sizeof(T) == sizeof(double), 1, hp);
        if (rc) return rc;
    }
    if (hd) {
        T *dl = tmpf<T>(c, 0);
        op_hdiv<T>(d, c->st, c->D(), tf<T>(c->svel), dl);
        c->launches += 1;
        xyi<T>(c, dl, dl);
        int rc = download(c, dl, sizeof(T) == sizeof(double), 1, hd);
        if (rc) return rc;
    }
    return PS3D_OK;
}

// kinetic-energy shell spectrum (genspec.f90:42-123) of the current vel
template <typename T> int ke_spectrum(ps3d_gpu_ctx *c, int nmax, double *spec, int *nbins, double *dk_out)
{
    const Dims &d = c->d;
    const long long N = d.nfield;
    int kmax = 0;
    for (int kx = 0; kx < d.nx; ++kx)
        for (int ky = 0; ky < d.ny; ++ky)
            for (int kz = 0; kz <= d.nz; ++kz) {
                const int km = (int)std::lround(std::sqrt(c->h_rkx[kx] * c->h_rkx[kx] + c->h_rky[ky] * c->h_rky[ky] +
                                                          c->h_rkz[kz] * c->h_rkz[kz]));
                kmax = km > kmax ? km : kmax;
            }
    const double dk = (double)kmax / std::sqrt((0.5 * d.nx) * (0.5 * d.nx) + (0.5 * d.ny) * (0.5 * d.ny) +
                                               (double)d.nz * d.nz);
    const int nb = kmax + 1;
    if (!c->spec_buf) {
        if (!dalloc(c, &c->spec_buf, (size_t)(d.nx + d.ny + 2 * nb) * sizeof(double)))
            return fail(c, PS3D_ERR_OUT_OF_MEMORY, "ke_spectrum: device allocation failed");
        cudaMemcpyAsync(c->spec_buf, c->h_rkx.data(), d.nx * sizeof(double), cudaMemcpyHostToDevice, c->st);
        cudaMemcpyAsync(c->spec_buf + d.nx, c->h_rky.data(), d.ny * sizeof(double), cudaMemcpyHostToDevice, c->st);
    }
    double *bins = c->spec_buf + d.nx + d.ny;
    unsigned long long *cnt = reinterpret_cast<unsigned long long *>(bins + nb);
    cudaMemsetAsync(bins, 0, 2 * (size_t)nb * sizeof(double), c->st);
    T *f = tmpf<T>(c, 0);
    for (int k = 0; k < 3; ++k) xyf<T>(c, tf<T>(c->vel) + k * N, f + k * N);
    col<T>(c, COL_DCT, f, f);
    col<T>(c, COL_DCT, f + N, f + N);
    col<T>(c, COL_DST, f + 2 * N, f + 2 * N);
    op_spec_bins<T>(d, c->st, c->spec_buf, c->spec_buf + d.nx, c->rkz, f, 1.0 / dk, kmax, bins, cnt);
    c->launches += 1;
    std::vector<double> hb(nb);
    std::vector<unsigned long long> hc(nb);
    cudaMemcpyAsync(hb.data(), bins, nb * sizeof(double), cudaMemcpyDeviceToHost, c->st);
    cudaMemcpyAsync(hc.data(), cnt, nb * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->st);
    double r1[RED1_N];
    int rc = energy<T>(c, r1);  // synchronises
    if (rc) return rc;
    const double ke = 0.5 * r1[2] * c->ncelli;
    const double pi = 3.14159265358979323846;
    const double pref = 4.0 / 3.0 * pi * dk * dk * dk;
    double tot = 0.0;
    for (int b = 0; b < nb; ++b) {
        if (hc[b] > 0)
            hb[b] = hb[b] * pref * (double)((long long)(b + 1) * (b + 1) * (b + 1) - (long long)b * b * b) /
                    (double)hc[b];
        tot += hb[b] * dk;
    }
    const double snorm = ke / tot;
    for (int b = 0; b < nb && b < nmax; ++b) spec[b] = hb[b] * snorm;
    *nbins = nb;
    *dk_out = dk;
    return PS3D_OK;
}

// setup_fields (utils.f90:136-184)
template <typename T> int setup_fields(ps3d_gpu_ctx *c, const double *vor_phys, const double *pert, double *te,
                                       double *en)
{
    const Dims &d = c->d;
    const long long N = d.nfield;
    // field_decompose_physical x3 in FP64 for both forms (the initial state
    // carries no FP32 rounding)
    int rc = upload(c, vor_phys, 3, c->svori, true);
    if (rc) return rc;
    for (int k = 0; k < 3; ++k) {
        xy_forward<double>(d, c->st, c->svori + k * N, c->svori + k * N, c->twx64, c->twy64, nullptr);
        columns<double>(d, c->st, COL_DECOMP, c->svori + k * N, c->svor + k * N, c->phim64, c->phip64,
                        c->twz2_64, nullptr);
        c->launches += 3;
    }
    if (pert) {
        rc = upload(c, pert, 3, c->svori, true);  // svori is free scratch here
        if (rc) return rc;
        op_add<double, double>(d, c->st, c->svor, c->svori, 3 * N);
        c->launches += 1;
    }
    op_mean_fix(d, c->st, c->svor, c->dstsum, c->fnzi, c->ini, c->savg, 0);
    cudaMemcpyAsync(c->ini, c->savg, 2 * sizeof(double), cudaMemcpyDeviceToDevice, c->st);
    cudaMemcpyAsync(c->ini_vor_mean, c->savg, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->st);
    c->launches += 1;
    if (sizeof(T) == sizeof(float)) project_state_mixed(c);
    rc = vor2vel<T>(c);
    if (rc) return rc;
    double r1[RED1_N];
    rc = energy<T>(c, r1);
    if (rc) return rc;
    double ke = 0.5 * r1[2] * c->ncelli, ens = 0.5 * r1[1] * c->ncelli;
    if (c->cfg.buoyancy) {
        // te = ke + ape, en = enstrophy + buoyancy-gradient integral
        // (utils.f90:169-180)
        double bd[4];
        rc = buoyancy_diagnostics<T>(c, bd);
        if (rc) return rc;
        ke = ke + bd[0];
        ens = ens + bd[1];
    }
    if (te) *te = ke;
    if (en) *en = ens;
    return ps3d_gpu_init_diffusion(c, ke, ens);
}

// buoyancy part of setup_fields (utils.f90:149-159): N^2 of the basic state
// unless given (calculate_basic_reference_state, physics.f90:310-340), the
// basic state N^2 z removed and the perturbation decomposed in FP64
template <typename T> int setup_buoyancy(ps3d_gpu_ctx *c, const double *buoy_phys)
{
    const Dims &d = c->d;
    if (!c->cfg.bfsq_given) {
        double sum = 0.0;
        const size_t nz1 = (size_t)d.nz + 1;
        for (long long col = 0; col < d.ncol; ++col) sum += buoy_phys[col * nz1 + d.nz] - buoy_phys[col * nz1];
        c->bfsq = sum / ((double)d.nx * (double)d.ny * c->cfg.extent[2]);
    }
    for (int iz = 0; iz <= d.nz; ++iz) c->h_bbarz[iz] = c->bfsq * (c->cfg.lower[2] + (double)iz * c->dx[2]);
    cudaMemcpyAsync(c->bprof, c->h_bbarz.data(), (d.nz + 1) * sizeof(double), cudaMemcpyHostToDevice, c->st);
    double *scratch = c->svori;  // FP64 scratch before the vorticity set-up
    int rc = upload(c, buoy_phys, 1, scratch, true);
    if (rc) return rc;
    op_sub_zprof(d, c->st, scratch, c->bprof);
    xy_forward<double>(d, c->st, scratch, scratch, c->twx64, c->twy64, nullptr);
    columns<double>(d, c->st, COL_DECOMP, scratch, c->sbuoy, c->phim64, c->phip64, c->twz2_64, nullptr);
    c->launches += 4;
    cudaMemsetAsync(c->sbuoys, 0, d.nfield * sizeof(T), c->st);
    if (c->bsm) cudaMemsetAsync(c->bsm, 0, d.nfield * sizeof(double), c->st);
    refresh_b32(c);
    return check(c, "setup_buoyancy");
}

template <typename T> int field_op(ps3d_gpu_ctx *c, int op, const double *in, double *out)
{
    const Dims &d = c->d;
    T *a = tmpf<T>(c, 4), *b = tmpf<T>(c, 5);
    int rc = upload(c, in, 1, a, c->fp64);
    if (rc) return rc;
    T *res = b;
    switch (op) {
    case PS3D_OP_FFTXYP2S: xyf<T>(c, a, b); break;
    case PS3D_OP_FFTXYS2P: xyi<T>(c, a, b); break;
    case PS3D_OP_DIFFX: op_diff<T>(d, c->st, c->D(), 0, a, b); c->launches += 1; break;
    case PS3D_OP_DIFFY: op_diff<T>(d, c->st, c->D(), 1, a, b); c->launches += 1; break;
    case PS3D_OP_FFTSINE: col<T>(c, COL_DST, a, b); break;
    case PS3D_OP_FFTCOSINE: col<T>(c, COL_DCT, a, b); break;
    case PS3D_OP_CENTRAL_DIFFZ: op_diffz<T>(d, c->st, c->dzi, a, b); c->launches += 1; break;
    case PS3D_OP_DECOMPOSE_SEMI: col<T>(c, COL_DECOMP, a, b); break;
    case PS3D_OP_COMBINE_SEMI: col<T>(c, COL_COMBINE, a, b); break;
    case PS3D_OP_DECOMPOSE_PHYS: xyf<T>(c, a, b); col<T>(c, COL_DECOMP, b, b); break;
    case PS3D_OP_COMBINE_PHYS: col<T>(c, COL_COMBINE, a, a); xyi<T>(c, a, b); break;
    case PS3D_OP_DIFFZ:
        if (!c->cfg.buoyancy) return fail(c, PS3D_ERR_INVALID_ARG, "field_op: diffz needs a buoyancy context");
        diffz_semi<T>(c, a, b, tmpf<T>(c, 3));
        col<T>(c, COL_DECOMP, b, b);
        break;
    default: return fail(c, PS3D_ERR_INVALID_ARG, "field_op: unknown op");
    }
    rc = check(c, "field_op");
    if (rc) return rc;
    return download(c, res, c->fp64, 1, out);
}

// --------------------------------------------------------- table set-up
void host_tables(ps3d_gpu_ctx *c)
{
    const Dims &d = c->d;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const double pi = acos(-1.0);
    std::vector<double> hrkx(nx + 1), hrky(ny + 1);
    for (int k = 1; k <= nx; ++k) hrkx[k] = (pi / c->cfg.extent[0]) * (double)k;
    for (int k = 1; k <= ny; ++k) hrky[k] = (pi / c->cfg.extent[1]) * (double)k;
    c->h_rkx.assign(nx, 0.0);
    c->h_rky.assign(ny, 0.0);
    c->h_rkz.assign(nz + 1, 0.0);
    const int nwx = nx / 2, nwy = ny / 2;
    for (int k = 1; k < nwx; ++k) c->h_rkx[k] = c->h_rkx[nx - k] = hrkx[2 * k];
    c->h_rkx[nwx] = hrkx[nx];
    for (int k = 1; k < nwy; ++k) c->h_rky[k] = c->h_rky[ny - k] = hrky[2 * k];
    c->h_rky[nwy] = hrky[ny];
    for (int i = 1; i <= nz; ++i) c->h_rkz[i] = (pi / c->cfg.extent[2]) * (double)i;
    // derivative coefficients (diffx/diffy, sta3dfft.f90:304-377)
    std::vector<double> hcx(nx, 0.0), hcy(ny, 0.0);
    for (int k = 1; k < nx; ++k) {
        const int dk = (2 * k < 2 * (nx - k)) ? 2 * k : 2 * (nx - k);
        hcx[k] = ((k >= nwx + 1) ? 1.0 : -1.0) * hrkx[dk];
    }
    if (nx % 2 == 0) hcx[nwx] = 0.0;
    for (int k = 1; k < ny; ++k) {
        const int dk = (2 * k < 2 * (ny - k)) ? 2 * k : 2 * (ny - k);
        hcy[k] = ((k >= nwy + 1) ? 1.0 : -1.0) * hrky[dk];
    }
    if (ny % 2 == 0) hcy[nwy] = 0.0;
    // k2l2, k2l2i (inversion_utils.f90:243-258)
    const size_t P2 = (size_t)nx * ny;
    c->h_k2l2.assign(P2, 0.0);
    c->h_k2l2i.assign(P2, 0.0);
    for (int kx = 0; kx < nx; ++kx)
        for (int ky = 0; ky < ny; ++ky)
            c->h_k2l2[ky + (size_t)ny * kx] = c->h_rkx[kx] * c->h_rkx[kx] + c->h_rky[ky] * c->h_rky[ky];
    c->h_k2l2[0] = 1.0;
    for (size_t i = 0; i < P2; ++i) c->h_k2l2i[i] = 1.0 / c->h_k2l2[i];
    c->h_k2l2[0] = 0.0;
    c->h_k2l2i[0] = 0.0;
    // filter (inversion_utils.f90:377-455): filt(kz,ky,kx) = filt0(ky,kx) * fz(kz)
    auto ipow = [](double x, int p) {
        double r = 1.0, b = x;
        while (p) {
            if (p & 1) r *= b;
            b *= b;
            p >>= 1;
        }
        return r;
    };
    double rkxmax = 0, rkymax = 0, rkzmax = 0;
    for (double v : c->h_rkx) rkxmax = fmax(rkxmax, v);
    for (double v : c->h_rky) rkymax = fmax(rkymax, v);
    for (double v : c->h_rkz) rkzmax = fmax(rkzmax, v);
    std::vector<double> skx(nx), sky(ny), skz(nz + 1);
    c->h_filt0.assign(P2, 0.0);
    c->h_fz.assign(nz + 1, 1.0);
    if (c->cfg.filtering == PS3D_TWO_THIRDS) {
        const double f23 = 2.0 / 3.0;
        for (int i = 0; i < nx; ++i) skx[i] = (c->h_rkx[i] <= f23 * rkxmax) ? 1.0 : 0.0;
        for (int i = 0; i < ny; ++i) sky[i] = (c->h_rky[i] <= f23 * rkymax) ? 1.0 : 0.0;
        for (int i = 0; i <= nz; ++i) skz[i] = (c->h_rkz[i] <= f23 * rkzmax) ? 1.0 : 0.0;
        for (int kx = 0; kx < nx; ++kx)
            for (int ky = 0; ky < ny; ++ky) c->h_filt0[ky + (size_t)ny * kx] = skx[kx] * sky[ky];
        for (int kz = 1; kz < nz; ++kz) c->h_fz[kz] = skz[kz];
    } else {
        const double kxmaxi = 1.0 / rkxmax, kymaxi = 1.0 / rkymax, kzmaxi = 1.0 / rkzmax;
        for (int i = 0; i < nx; ++i) skx[i] = -36.0 * ipow(kxmaxi * c->h_rkx[i], 36);
        for (int i = 0; i < ny; ++i) sky[i] = -36.0 * ipow(kymaxi * c->h_rky[i], 36);
        for (int i = 0; i <= nz; ++i) skz[i] = -36.0 * ipow(kzmaxi * c->h_rkz[i], 36);
        for (int kx = 0; kx < nx; ++kx)
            for (int ky = 0; ky < ny; ++ky) c->h_filt0[ky + (size_t)ny * kx] = exp(skx[kx] + sky[ky]);
        for (int kz = 1; kz < nz; ++kz) c->h_fz[kz] = exp(skz[kz]);
    }
    c->h_filt0[0] = 1.0;
    // z tables
    std::vector<double> hrkzi(nz + 1, 0.0), zm(nz + 1), zp(nz + 1), dstsum(nz + 1, 0.0), dctcos(2 * nz);
    for (int i = 1; i < nz; ++i) hrkzi[i] = 1.0 / c->h_rkz[i];
    const double lower = c->cfg.lower[2], upper = c->cfg.lower[2] + c->cfg.extent[2];
    for (int iz = 0; iz <= nz; ++iz) {
        const double z = lower + c->dx[2] * (double)iz;
        zm[iz] = upper - z;
        zp[iz] = z - lower;
    }
    c->h_gamtop.assign(nz + 1, 0.0);
    c->h_gambot.assign(nz + 1, 0.0);
    for (int iz = 0; iz <= nz; ++iz) {
        const double php = zp[iz] / c->cfg.extent[2];
        c->h_gamtop[iz] = 0.5 * c->cfg.extent[2] * (php * php - 1.0 / 3.0);
    }
    for (int iz = 0; iz <= nz; ++iz) c->h_gambot[iz] = c->h_gamtop[nz - iz];
    const double sq = sqrt(2.0 / (double)nz);
    for (int j = 1; j < nz; ++j) {
        double s = 0.0;
        for (int k = 1; k < nz; ++k) s += sin(pi * (double)(((long long)j * k) % (2 * nz)) / (double)nz);
        dstsum[j] = sq * s;
    }
    for (int m = 0; m < 2 * nz; ++m) dctcos[m] = cos(pi * (double)m / (double)nz);

    auto up = [&](double *dst, const std::vector<double> &v) {
        cudaMemcpyAsync(dst, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, c->st);
    };
    up(c->cx, hcx);
    up(c->cy, hcy);
    up(c->k2l2, c->h_k2l2);
    up(c->k2l2i, c->h_k2l2i);
    up(c->filt0, c->h_filt0);
    up(c->fz, c->h_fz);
    up(c->rkz, c->h_rkz);
    up(c->rkzi, hrkzi);
    up(c->gamtop, c->h_gamtop);
    up(c->gambot, c->h_gambot);
    up(c->dstsum, dstsum);
    up(c->dctcos, dctcos);
    up(c->zm, zm);
    up(c->zp, zp);
    cudaStreamSynchronize(c->st);  // host vectors go out of scope
}

template <typename T> void twiddles(ps3d_gpu_ctx *c, void *dst, int n)
{
    std::vector<CT<T>> tw(n);
    for (int k = 0; k < n; ++k) {
        // exact at multiples of pi/2
        double s = sin(2.0 * M_PI * (double)k / (double)n), co = cos(2.0 * M_PI * (double)k / (double)n);
        if (4 * k % n == 0) {
            const int q = 4 * k / n;
            co = (q == 0) ? 1.0 : (q == 2 ? -1.0 : 0.0);
            s = (q == 1) ? 1.0 : (q == 3 ? -1.0 : 0.0);
        }
        tw[k].x = (decltype(tw[k].x))co;
        tw[k].y = (decltype(tw[k].y))(-s);
    }
    cudaMemcpyAsync(dst, tw.data(), n * sizeof(CT<T>), cudaMemcpyHostToDevice, c->st);
    cudaStreamSynchronize(c->st);
}

// Autotuner of the FP32 line FFTs: where a line length has more than one
// kernel shape (lines32_has_shape), every pass (forward / inverse, y / x)
// is timed with each shape on a zeroed scratch field (one warm-up and five
// timed launches, CUDA events) and keeps the fastest.
int autotune_lines(ps3d_gpu_ctx *c)
{
    Dims &d = c->d;
    if (lines32_shapes(d.nx) < 2 && lines32_shapes(d.ny) < 2) return PS3D_OK;
    float *a = tmpf<float>(c, 0), *b = tmpf<float>(c, 1);
    cudaMemsetAsync(a, 0, d.nfield * sizeof(float), c->st);
    const float2 *twx = tf<float2>(c->twx), *twy = tf<float2>(c->twy);
    for (int pass = 0; pass < 4; ++pass) {
        const bool inv = pass >= 2, xl = (pass & 1) != 0;
        const int n = xl ? d.nx : d.ny;
        const int ns = lines32_shapes(n);
        if (ns < 2) continue;
        const long long ls = xl ? (long long)d.ny * d.P : d.P, nb = xl ? d.ny : d.nx,
                        bs = xl ? d.P : (long long)d.ny * d.P;
        // five timed launches per shape after one warm-up; the TMA-fed
        // kernel (shape 2) replaces the best block shape only if it is at
        // least 5% faster, so timing noise does not flip the choice
        int best = 0;
        for (int w = 0; w < 3; ++w) {
            if (!lines32_has_shape(n, w)) continue;
            launch_lines32(c->st, a, b, n, d.P, d.nz + 1, ls, nb, bs, inv, xl ? twx : twy, w);
            cudaEventRecord(c->ev0, c->st);
            for (int r = 0; r < 5; ++r) launch_lines32(c->st, a, b, n, d.P, d.nz + 1, ls, nb, bs, inv, xl ? twx : twy, w);
            cudaEventRecord(c->ev1, c->st);
            const int rc = sync_check(c, "autotune");
            if (rc) return rc;
            float f = 0.0f;
            cudaEventElapsedTime(&f, c->ev0, c->ev1);
            c->tune_ms[pass][w] = f / 5.0;
            const double margin = (w == 2) ? 0.95 : 1.0;
            if (c->tune_ms[pass][w] < margin * c->tune_ms[pass][best]) best = w;
        }
        d.line_shape[pass] = (signed char)best;
    }
    return PS3D_OK;
}

template <typename T> int allocate_fields(ps3d_gpu_ctx *c)
{
    const Dims &d = c->d;
    const size_t N = (size_t)d.nfield;
    const size_t fb = N * sizeof(T), f64 = N * sizeof(double);
    bool ok = dalloc(c, &c->svor, 3 * f64) && dalloc(c, &c->svori, 3 * f64) && dalloc(c, &c->svorf, 3 * f64) &&
              dalloc(c, &c->vor, 3 * fb) && dalloc(c, &c->vel, 3 * fb) && dalloc(c, &c->svel, 3 * fb) &&
              dalloc(c, &c->svorts, 3 * fb) && dalloc(c, &c->tmp, NTMP * fb) && dalloc(c, &c->phim, fb) &&
              dalloc(c, &c->phip, fb) && dalloc(c, &c->thetam, fb) && dalloc(c, &c->thetap, fb) &&
              dalloc(c, &c->dthetam, fb) && dalloc(c, &c->dthetap, fb) && dalloc(c, &c->green, fb);
    if (ok && c->cfg.stepper == PS3D_CN2) ok = dalloc(c, &c->vortsm, 3 * f64);
    // the mixed form holds es beside the three tendency components
    if (ok && c->cfg.hold_source) ok = dalloc(c, &c->held, (c->fp64 ? 3 : 4) * fb);
    if (ok && c->cfg.buoyancy) {
        const size_t P2b = (size_t)d.ncol * sizeof(double);
        ok = dalloc(c, &c->sbuoy, f64) && dalloc(c, &c->sbuoyi, f64) && dalloc(c, &c->sbuoyf, f64) &&
             dalloc(c, &c->buoy, fb) && dalloc(c, &c->sbuoys, fb) && dalloc(c, &c->dphim, fb) &&
             dalloc(c, &c->dphip, fb) && dalloc(c, &c->bhdis, P2b) && dalloc(c, &c->bdiss, P2b) &&
             dalloc(c, &c->bpq, P2b) && dalloc(c, &c->bmq, P2b) && dalloc(c, &c->bpq2, P2b) &&
             dalloc(c, &c->bmq2, P2b) && dalloc(c, &c->bpart, (size_t)bdiag_blocks(d) * 4 * sizeof(double)) &&
             dalloc(c, &c->bres, 4 * sizeof(double)) && dalloc(c, &c->bprof, (d.nz + 1) * sizeof(double)) &&
             dalloc(c, &c->bmax, sizeof(unsigned long long));
        if (ok && c->cfg.stepper == PS3D_CN2) ok = dalloc(c, &c->bsm, f64);
        if (ok && c->cfg.hold_source) ok = dalloc(c, &c->heldb, fb);
        if (ok && !c->fp64) ok = dalloc(c, &c->sbuoy32, N * sizeof(float));
        if (ok) {
            cudaMemsetAsync(c->sbuoy, 0, f64, c->st);
            cudaMemsetAsync(c->buoy, 0, fb, c->st);
            cudaMemsetAsync(c->sbuoys, 0, fb, c->st);
            if (c->sbuoy32) cudaMemsetAsync(c->sbuoy32, 0, N * sizeof(float), c->st);
        }
    }
    if (ok && !c->fp64)
        ok = dalloc(c, &c->svor32, 3 * N * sizeof(float)) && dalloc(c, &c->es_src, N * sizeof(float)) &&
             dalloc(c, &c->mf64, 2 * (size_t)d.P * sizeof(double)) &&
             dalloc(c, &c->twz32, d.nz * sizeof(float2)) && dalloc(c, &c->sinz32, d.nz * sizeof(float)) &&
             dalloc(c, &c->cosz32, d.nz * sizeof(float)) &&
             dalloc(c, &c->stage64, f64) && dalloc(c, &c->phim64, f64) && dalloc(c, &c->phip64, f64) &&
             dalloc(c, &c->twx64, d.nx * sizeof(double2)) && dalloc(c, &c->twy64, d.ny * sizeof(double2)) &&
             dalloc(c, &c->twz2_64, 2 * d.nz * sizeof(double2));
    const size_t P2 = (size_t)d.ncol * sizeof(double), Z = (size_t)(d.nz + 1) * sizeof(double);
    ok = ok && dalloc(c, &c->twx, d.nx * sizeof(CT<T>)) && dalloc(c, &c->twy, d.ny * sizeof(CT<T>)) &&
         dalloc(c, &c->twz2, 2 * d.nz * sizeof(CT<T>));
    ok = ok && dalloc(c, &c->k2l2, P2) && dalloc(c, &c->k2l2i, P2) && dalloc(c, &c->filt0, P2) &&
         dalloc(c, &c->vhdis, P2) && dalloc(c, &c->vdiss, P2) && dalloc(c, &c->epq, P2) && dalloc(c, &c->emq, P2) &&
         dalloc(c, &c->epq2, P2) && dalloc(c, &c->emq2, P2);
    ok = ok && dalloc(c, &c->fz, Z) && dalloc(c, &c->rkz, Z) && dalloc(c, &c->rkzi, Z) && dalloc(c, &c->gamtop, Z) &&
         dalloc(c, &c->gambot, Z) && dalloc(c, &c->dstsum, Z) && dalloc(c, &c->dctcos, 2 * d.nz * sizeof(double)) &&
         dalloc(c, &c->cx, d.nx * sizeof(double)) && dalloc(c, &c->cy, d.ny * sizeof(double)) &&
         dalloc(c, &c->zm, Z) && dalloc(c, &c->zp, Z) && dalloc(c, &c->ubar, Z) && dalloc(c, &c->vbar, Z) &&
         dalloc(c, &c->ini, 2 * sizeof(double)) && dalloc(c, &c->savg, 2 * sizeof(double)) &&
         dalloc(c, &c->part, (size_t)red_nblocks(d) * RED1_N * sizeof(double)) &&
         dalloc(c, &c->res1, RED1_N * sizeof(double)) && dalloc(c, &c->res2, RED2_N * sizeof(double)) &&
         dalloc(c, &c->flag, sizeof(int)) && dalloc(c, &c->flag_chk, sizeof(int)) && dalloc(c, &c->sc, sizeof(StepScal)) &&
         dalloc(c, &c->roll_dev, c->roll.hist.size() * sizeof(double));
    if (!ok) return fail(c, PS3D_ERR_OUT_OF_MEMORY, "device allocation failed");
    twiddles<T>(c, c->twx, d.nx);
    twiddles<T>(c, c->twy, d.ny);
    twiddles<T>(c, c->twz2, 2 * d.nz);
    if (c->fp64) {
        c->twx64 = tf<double2>(c->twx);
        c->twy64 = tf<double2>(c->twy);
        c->twz2_64 = tf<double2>(c->twz2);
        c->phim64 = tf<double>(c->phim);
        c->phip64 = tf<double>(c->phip);
    } else {
        twiddles<double>(c, c->twx64, d.nx);
        twiddles<double>(c, c->twy64, d.ny);
        twiddles<double>(c, c->twz2_64, 2 * d.nz);
        twiddles<float>(c, c->twz32, d.nz);
        std::vector<float> sn(d.nz), cs(d.nz);
        for (int j = 0; j < d.nz; ++j) {
            sn[j] = (float)sin(M_PI * (double)j / (double)d.nz);
            cs[j] = (float)cos(M_PI * (double)j / (double)d.nz);
        }
        cudaMemcpyAsync(c->sinz32, sn.data(), d.nz * sizeof(float), cudaMemcpyHostToDevice, c->st);
        cudaMemcpyAsync(c->cosz32, cs.data(), d.nz * sizeof(float), cudaMemcpyHostToDevice, c->st);
        cudaStreamSynchronize(c->st);
    }
    host_tables(c);
    op_hyperbolic_tables<T>(d, c->st, c->k2l2, c->k2l2i, c->rkz, c->zm, c->zp, c->cfg.extent[2], tf<T>(c->phim),
                            tf<T>(c->phip), tf<T>(c->thetam), tf<T>(c->thetap), tf<T>(c->dthetam),
                            tf<T>(c->dthetap), tf<T>(c->green));
    c->launches += 1;
    if (c->cfg.buoyancy) {
        op_dphi_tables<T>(d, c->st, c->k2l2, c->zm, c->zp, c->cfg.extent[2], tf<T>(c->dphim), tf<T>(c->dphip));
        c->launches += 1;
        c->h_bbarz.assign(d.nz + 1, 0.0);
        for (int iz = 0; iz <= d.nz; ++iz) c->h_bbarz[iz] = c->bfsq * (c->cfg.lower[2] + (double)iz * c->dx[2]);
    }
    if (!c->fp64) {
        // FP64 harmonic functions for the FP64 set-up and projection; the
        // remaining FP64 outputs go to scratch (svori, svorf)
        double *s = c->svori, *s2 = c->svorf;
        op_hyperbolic_tables<double>(d, c->st, c->k2l2, c->k2l2i, c->rkz, c->zm, c->zp, c->cfg.extent[2],
                                     c->phim64, c->phip64, s, s + N, s + 2 * N, s2, s2 + N);
        c->launches += 1;
    }
    int rc = sync_check(c, "create");
    if (rc) return rc;
    return c->fp64 ? PS3D_OK : autotune_lines(c);
}

#define DISPATCH(c, fn, ...) ((c)->fp64 ? fn<double>(__VA_ARGS__) : fn<float>(__VA_ARGS__))

// The fused products kernel saves the products' trip through HBM; while a
// field fits comfortably in L2 (below 2^24 elements, 64 MB in FP32) there
// is nothing to save and the plain kernels run faster (the fused first pass
// reads four fields per output point).  PS3D_FUSE_PRODUCTS=1 or 0 in the
// environment forces the choice; both give bitwise the same tendency.
bool products_fused_default(const Dims &d)
{
    if (const char *e = getenv("PS3D_FUSE_PRODUCTS")) {
        if (e[0] == '1') return true;
        if (e[0] == '0') return false;
    }
    return d.nfield >= (1LL << 24);
}

int enter(ps3d_gpu_ctx *c)
{
    if (!c) return PS3D_ERR_INVALID_ARG;
    if (cudaSetDevice(c->cfg.device) != cudaSuccess) return check(c, "cudaSetDevice");
    return PS3D_OK;
}

}  // namespace

// ======================================================================
// public C ABI
// ======================================================================
extern "C" {

const char *ps3d_gpu_strerror(int status)
{
    switch (status) {
    case PS3D_OK: return "ok";
    case PS3D_ERR_INVALID_ARG: return "invalid argument";
    case PS3D_ERR_UNSUPPORTED_SIZE: return "unsupported grid size";
    case PS3D_ERR_CUDA: return "CUDA error";
    case PS3D_ERR_OUT_OF_MEMORY: return "device out of memory";
    case PS3D_ERR_NOT_READY: return "not ready (call init_diffusion/setup_fields first)";
    case PS3D_ERR_NONFINITE: return "non-finite value detected";
    case PS3D_ERR_DEVICE_LIMIT: return "bounded device loop reached its limit";
    case PS3D_ERR_NO_DEVICE: return "no suitable CUDA device";
    default: return "unknown status";
    }
}

const char *ps3d_gpu_last_error(const ps3d_gpu_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }

long long ps3d_gpu_device_bytes(const ps3d_gpu_ctx *ctx) { return ctx ? ctx->bytes : 0; }

long long ps3d_gpu_launch_count(const ps3d_gpu_ctx *ctx) { return ctx ? ctx->launches : 0; }

int ps3d_gpu_create(const ps3d_gpu_config *cfg, ps3d_gpu_ctx **out)
{
    if (!cfg || !out) return PS3D_ERR_INVALID_ARG;
    *out = nullptr;
    const int nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
    const int zmax = cfg->precision == PS3D_PRECISION_FP64 ? 1024 : 2048;
    // even lengths with factors 2, 3 and 5 only (the factorisation of
    // stafft.f90:128-187 with its radices 2..6)
    auto ok_len = [](int n, int lo, int hi) { return n >= lo && n <= hi && n % 2 == 0 && radix235(n); };
    if (!ok_len(nx, 8, 2048) || !ok_len(ny, 8, 2048) || !ok_len(nz, 8, zmax)) return PS3D_ERR_UNSUPPORTED_SIZE;
    if (cfg->precision != PS3D_PRECISION_FP64 && cfg->precision != PS3D_PRECISION_MIXED) return PS3D_ERR_INVALID_ARG;
    if (cfg->stepper != PS3D_IMPL_DIFF_RK4 && cfg->stepper != PS3D_CN2) return PS3D_ERR_INVALID_ARG;
    if (cfg->pretype < 0 || cfg->pretype > 6 || cfg->nnu < 1 || !(cfg->extent[0] > 0) || !(cfg->extent[1] > 0) ||
        !(cfg->extent[2] > 0))
        return PS3D_ERR_INVALID_ARG;
    // 'bfmax' / 'roll-mean-bfmax' need the buoyancy build (advance.f90:395-407)
    if (!cfg->buoyancy && cfg->pretype == PS3D_PRE_ROLL_MEAN_BFMAX) return PS3D_ERR_INVALID_ARG;
    if (cfg->buoyancy && (cfg->buoy_pretype < 0 || cfg->buoy_pretype > 6 || cfg->buoy_nnu < 1))
        return PS3D_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= cfg->device || cfg->device < 0) {
        cudaGetLastError();
        return PS3D_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, cfg->device) != cudaSuccess || prop.major != 10 || prop.minor != 3) {
        cudaGetLastError();
        return PS3D_ERR_NO_DEVICE;
    }
    ps3d_gpu_ctx *c = new ps3d_gpu_ctx();
    static std::atomic<unsigned long long> next_serial{0};
    c->serial = ++next_serial;
    c->cfg = *cfg;
    c->fp64 = cfg->precision == PS3D_PRECISION_FP64;
    cudaSetDevice(cfg->device);
    transforms_init();
    columns32_init();
    colz_init();
    cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
    cudaStreamCreateWithFlags(&c->st_chk, cudaStreamNonBlocking);
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);
    cudaEventCreateWithFlags(&c->ev_chk0, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->ev_chk, cudaEventDisableTiming);
    Dims &d = c->d;
    d.nx = nx;
    d.ny = ny;
    d.nz = nz;
    d.P = ((nz + 1) + 7) / 8 * 8;
    d.ncol = (long long)nx * ny;
    d.nfield = (long long)d.P * d.ncol;
    c->fuse_products = products_fused_default(d);
    const int nc[3] = {nx, ny, nz};
    for (int k = 0; k < 3; ++k) c->dx[k] = cfg->extent[k] / (double)nc[k];
    c->ncell = (long long)nx * ny * nz;
    c->ncelli = 1.0 / (double)c->ncell;
    c->fnzi = 1.0 / (double)nz;
    c->dzi = 1.0 / c->dx[2];
    c->roll.hist.assign(cfg->roll_mean_win_size > 0 ? cfg->roll_mean_win_size : 1000, 0.0);
    c->roll_b.hist.assign(cfg->buoy_roll_mean_win_size > 0 ? cfg->buoy_roll_mean_win_size : 1000, 0.0);
    c->bfsq = cfg->buoyancy ? cfg->bfsq : 0.0;
    const int rc = DISPATCH(c, allocate_fields, c);
    if (rc) {
        ps3d_gpu_destroy(c);
        return rc;
    }
    *out = c;
    return PS3D_OK;
}

int ps3d_gpu_destroy(ps3d_gpu_ctx *c)
{
    if (!c) return PS3D_OK;
    cudaSetDevice(c->cfg.device);
    if (c->st) cudaStreamSynchronize(c->st);
    if (c->closure) closure_detach(c->closure, c);
    if (c->graph) cudaGraphExecDestroy(c->graph);
    delete c->batch;
    for (void *p : c->allocs) cudaFree(p);
    if (c->probe.ev) {
        for (int i = 0; i < 2 * Probe::MAXP; ++i) cudaEventDestroy(c->probe.ev[i]);
        delete[] c->probe.ev;
    }
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->ev_chk0) cudaEventDestroy(c->ev_chk0);
    if (c->ev_chk) cudaEventDestroy(c->ev_chk);
    if (c->st_chk) {
        cudaStreamSynchronize(c->st_chk);
        cudaStreamDestroy(c->st_chk);
    }
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
    return PS3D_OK;
}

int ps3d_gpu_set_field(ps3d_gpu_ctx *c, int which, const double *host)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!host) return PS3D_ERR_INVALID_ARG;
    switch (which) {
    case PS3D_FIELD_SVOR:
        rc = upload(c, host, 3, c->svor, true);
        if (!rc && !c->fp64) project_state_mixed(c);
        break;
    case PS3D_FIELD_VOR: rc = upload(c, host, 3, c->vor, c->fp64); break;
    case PS3D_FIELD_VEL: rc = upload(c, host, 3, c->vel, c->fp64); break;
    case PS3D_FIELD_SVEL: rc = upload(c, host, 3, c->svel, c->fp64); break;
    case PS3D_FIELD_SVORTS: rc = upload(c, host, 3, c->svorts, c->fp64); break;
    case PS3D_FIELD_SBUOY:
    case PS3D_FIELD_BUOY:
    case PS3D_FIELD_SBUOYS:
        if (!c->cfg.buoyancy) return fail(c, PS3D_ERR_INVALID_ARG, "set_field: no buoyancy in this context");
        if (which == PS3D_FIELD_SBUOY) {
            rc = upload(c, host, 1, c->sbuoy, true);
            if (!rc) refresh_b32(c);
        } else {
            rc = upload(c, host, 1, which == PS3D_FIELD_BUOY ? c->buoy : c->sbuoys, c->fp64);
        }
        break;
    default: return fail(c, PS3D_ERR_INVALID_ARG, "set_field: unknown field");
    }
    if (rc) return rc;
    return sync_check(c, "set_field");
}

int ps3d_gpu_get_field(ps3d_gpu_ctx *c, int which, double *host)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!host) return PS3D_ERR_INVALID_ARG;
    switch (which) {
    case PS3D_FIELD_SVOR: return download(c, c->svor, true, 3, host);
    case PS3D_FIELD_VOR: return download(c, c->vor, c->fp64, 3, host);
    case PS3D_FIELD_VEL: return download(c, c->vel, c->fp64, 3, host);
    case PS3D_FIELD_SVEL: return download(c, c->svel, c->fp64, 3, host);
    case PS3D_FIELD_SVORTS: return download(c, c->svorts, c->fp64, 3, host);
    case PS3D_FIELD_SBUOY:
    case PS3D_FIELD_BUOY:
    case PS3D_FIELD_SBUOYS:
        if (!c->cfg.buoyancy) return fail(c, PS3D_ERR_INVALID_ARG, "get_field: no buoyancy in this context");
        if (which == PS3D_FIELD_SBUOY) return download(c, c->sbuoy, true, 1, host);
        return download(c, which == PS3D_FIELD_BUOY ? c->buoy : c->sbuoys, c->fp64, 1, host);
    default: return fail(c, PS3D_ERR_INVALID_ARG, "get_field: unknown field");
    }
}

int ps3d_gpu_set_ini_vor_mean(ps3d_gpu_ctx *c, const double v[2])
{
    int rc = enter(c);
    if (rc) return rc;
    c->ini_vor_mean[0] = v[0];
    c->ini_vor_mean[1] = v[1];
    cudaMemcpyAsync(c->ini, c->ini_vor_mean, 2 * sizeof(double), cudaMemcpyHostToDevice, c->st);
    return sync_check(c, "set_ini_vor_mean");
}

int ps3d_gpu_get_ini_vor_mean(ps3d_gpu_ctx *c, double v[2])
{
    int rc = enter(c);
    if (rc) return rc;
    rc = sync_check(c, "get_ini_vor_mean");
    v[0] = c->ini_vor_mean[0];
    v[1] = c->ini_vor_mean[1];
    return rc;
}

int ps3d_gpu_get_table(ps3d_gpu_ctx *c, int which, double *host)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!host) return PS3D_ERR_INVALID_ARG;
    const Dims &d = c->d;
    auto put = [&](const std::vector<double> &v) { memcpy(host, v.data(), v.size() * sizeof(double)); };
    std::vector<double> tmp;
    switch (which) {
    case 0: put(c->h_k2l2); return PS3D_OK;
    case 1: put(c->h_k2l2i); return PS3D_OK;
    case 2: {
        // filt(kz, ky, kx) = filt0 * fz, (0,0) column = 1
        const size_t nz1 = d.nz + 1;
        for (long long col = 0; col < d.ncol; ++col)
            for (int iz = 0; iz <= d.nz; ++iz)
                host[col * nz1 + iz] = (col == 0) ? 1.0 : c->h_filt0[col] * ((iz == 0 || iz == d.nz) ? 1.0 : c->h_fz[iz]);
        return PS3D_OK;
    }
    case 3: return download(c, c->green, c->fp64, 1, host);
    case 4: return download(c, c->phim, c->fp64, 1, host);
    case 5: return download(c, c->phip, c->fp64, 1, host);
    case 6: return download(c, c->thetam, c->fp64, 1, host);
    case 7: return download(c, c->thetap, c->fp64, 1, host);
    case 8: return download(c, c->dthetam, c->fp64, 1, host);
    case 9: return download(c, c->dthetap, c->fp64, 1, host);
    case 10: put(c->h_gamtop); return PS3D_OK;
    case 11: put(c->h_gambot); return PS3D_OK;
    case 12:
        cudaMemcpyAsync(host, c->vhdis, d.ncol * sizeof(double), cudaMemcpyDeviceToHost, c->st);
        return sync_check(c, "get_table");
    case 13: put(c->h_rkx); return PS3D_OK;
    case 14: put(c->h_rky); return PS3D_OK;
    case 15: put(c->h_rkz); return PS3D_OK;
    case 16:
    case 17:
    case 18:
    case 19:
        if (!c->cfg.buoyancy) return fail(c, PS3D_ERR_INVALID_ARG, "get_table: no buoyancy in this context");
        if (which == 16) return download(c, c->dphim, c->fp64, 1, host);
        if (which == 17) return download(c, c->dphip, c->fp64, 1, host);
        if (which == 19) {
            put(c->h_bbarz);
            return PS3D_OK;
        }
        cudaMemcpyAsync(host, c->bhdis, d.ncol * sizeof(double), cudaMemcpyDeviceToHost, c->st);
        return sync_check(c, "get_table");
    default: return fail(c, PS3D_ERR_INVALID_ARG, "get_table: unknown table");
    }
}

int ps3d_gpu_setup_fields(ps3d_gpu_ctx *c, const double *vor_phys, const double *pert, double *te, double *en)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!vor_phys) return PS3D_ERR_INVALID_ARG;
    if (c->cfg.buoyancy)
        return fail(c, PS3D_ERR_INVALID_ARG, "setup_fields: a buoyancy context needs ps3d_gpu_setup_fields_buoyancy");
    return DISPATCH(c, setup_fields, c, vor_phys, pert, te, en);
}

int ps3d_gpu_setup_fields_buoyancy(ps3d_gpu_ctx *c, const double *vor_phys, const double *pert,
                                   const double *buoy_phys, double *te, double *en)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!vor_phys) return PS3D_ERR_INVALID_ARG;
    if (!c->cfg.buoyancy) return DISPATCH(c, setup_fields, c, vor_phys, pert, te, en);
    if (!buoy_phys) return PS3D_ERR_INVALID_ARG;
    rc = DISPATCH(c, setup_buoyancy, c, buoy_phys);
    if (rc) return rc;
    return DISPATCH(c, setup_fields, c, vor_phys, pert, te, en);
}

int ps3d_gpu_buoyancy_params(ps3d_gpu_ctx *c, double *bfsq, double *bvisc)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!c->cfg.buoyancy) return fail(c, PS3D_ERR_INVALID_ARG, "buoyancy_params: no buoyancy in this context");
    if (bfsq) *bfsq = c->bfsq;
    if (bvisc) *bvisc = c->bvisc;
    return PS3D_OK;
}

int ps3d_gpu_buoyancy_diagnostics(ps3d_gpu_ctx *c, double out[4])
{
    int rc = enter(c);
    if (rc) return rc;
    if (!out) return PS3D_ERR_INVALID_ARG;
    if (!c->cfg.buoyancy) return fail(c, PS3D_ERR_INVALID_ARG, "buoyancy_diagnostics: no buoyancy in this context");
    return DISPATCH(c, buoyancy_diagnostics, c, out);
}

// init_diffusion (inversion_utils.f90:124-218)
int ps3d_gpu_init_diffusion(ps3d_gpu_ctx *c, double te, double en)
{
    int rc = enter(c);
    if (rc) return rc;
    double rkxmax = 0.0, rkymax = 0.0;
    for (double v : c->h_rkx) rkxmax = fmax(rkxmax, v);
    for (double v : c->h_rky) rkymax = fmax(rkymax, v);
    const double km = fmax(rkxmax, rkymax);
    const double k2max = km * km;
    const double rkmsi = 1.0 / k2max;
    const int p = c->cfg.nnu;
    auto ipow = [](double x, int e) {
        double r = 1.0, b = x;
        while (e) {
            if (e & 1) r *= b;
            b *= b;
            e >>= 1;
        }
        return r;
    };
    // get_viscosity (:157-185) and init_dissipation (:189-218)
    auto viscosity = [&](int scale, double prediss, int pp) {
        if (scale == PS3D_GEOPHYSICAL) return prediss * ipow(rkmsi, pp);
        return prediss * pow(k2max * te / en, 1.0 / 3.0) * ipow(rkmsi, pp);
    };
    auto dissipation = [&](double vis, int pp, double *dst) {
        std::vector<double> h(c->d.ncol);
        for (long long i = 0; i < c->d.ncol; ++i) h[i] = (pp == 1) ? vis * c->h_k2l2[i] : vis * ipow(c->h_k2l2[i], pp);
        cudaMemcpyAsync(dst, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c->st);
        cudaStreamSynchronize(c->st);
    };
    c->vvisc = viscosity(c->cfg.length_scale, c->cfg.prediss, p);
    dissipation(c->vvisc, p, c->vhdis);
    if (c->cfg.buoyancy) {
        c->bvisc = viscosity(c->cfg.buoy_length_scale, c->cfg.buoy_prediss, c->cfg.buoy_nnu);
        dissipation(c->bvisc, c->cfg.buoy_nnu, c->bhdis);
    }
    rc = sync_check(c, "init_diffusion");
    if (rc) return rc;
    c->diffusion_ready = true;
    return PS3D_OK;
}

int ps3d_gpu_vor2vel(ps3d_gpu_ctx *c)
{
    int rc = enter(c);
    if (rc) return rc;
    rc = DISPATCH(c, vor2vel, c);
    if (rc) return rc;
    return sync_check(c, "vor2vel");
}

int ps3d_gpu_source(ps3d_gpu_ctx *c)
{
    int rc = enter(c);
    if (rc) return rc;
    c->closure_fresh = true;
    rc = DISPATCH(c, source, c);
    if (rc) return rc;
    return sync_check(c, "source");
}

int ps3d_gpu_set_closure(ps3d_gpu_ctx *c, ps3d_closure *cl, int flags)
{
    int rc = enter(c);
    if (rc) return rc;
    if (flags & ~(PS3D_CLOSURE_EVERY_STAGE | PS3D_CLOSURE_CLIP | PS3D_CLOSURE_WALLS)) return PS3D_ERR_INVALID_ARG;
    cudaStreamSynchronize(c->st);
    if (cl) {
        std::string e;
        rc = closure_attach(cl, c, c->d.nx, c->d.ny, c->d.nz, c->cfg.device, &e);
        if (rc) return fail(c, rc, e);
        if (!c->corr) {
            const size_t bytes = 3 * (size_t)c->d.nfield * (c->fp64 ? sizeof(double) : sizeof(float));
            if (!dalloc(c, &c->corr, bytes)) {
                closure_detach(cl, c);
                return fail(c, PS3D_ERR_OUT_OF_MEMORY, "closure correction fields");
            }
            cudaMemsetAsync(c->corr, 0, bytes, c->st);
        }
    }
    if (c->closure && c->closure != cl) closure_detach(c->closure, c);
    c->closure = cl;
    c->closure_flags = flags;
    c->closure_fresh = true;
    // a captured step holds the launches of the previous configuration
    if (c->graph) {
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
    }
    return sync_check(c, "set_closure");
}

int ps3d_gpu_adapt(ps3d_gpu_ctx *c, double t, double *dt, ps3d_gpu_diag *diag)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!dt) return PS3D_ERR_INVALID_ARG;
    if (!c->diffusion_ready) return fail(c, PS3D_ERR_NOT_READY, "adapt before init_diffusion");
    return DISPATCH(c, adapt, c, t, dt, diag);
}

int ps3d_gpu_set_diffusion(ps3d_gpu_ctx *c, double dt, double pref)
{
    return ps3d_gpu_set_diffusion_vb(c, dt, pref, 0.0);
}

int ps3d_gpu_set_diffusion_vb(ps3d_gpu_ctx *c, double dt, double vpref, double bpref)
{
    int rc = enter(c);
    if (rc) return rc;
    rc = set_diffusion(c, dt, vpref, bpref);
    if (rc) return rc;
    return sync_check(c, "set_diffusion");
}

int ps3d_gpu_step(ps3d_gpu_ctx *c, double *t, double dt)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!t) return PS3D_ERR_INVALID_ARG;
    rc = DISPATCH(c, step, c, t, dt);
    if (rc) return rc;
    return sync_check(c, "step");
}

int ps3d_gpu_advance(ps3d_gpu_ctx *c, double *t, int nsteps, ps3d_gpu_diag *diag)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!t || nsteps < 0) return PS3D_ERR_INVALID_ARG;
    if (!c->diffusion_ready) return fail(c, PS3D_ERR_NOT_READY, "advance before init_diffusion");
    for (int s = 0; s < nsteps; ++s) {
        rc = DISPATCH(c, advance, c, t, diag ? diag + s : nullptr);
        if (rc) return rc;
    }
    return sync_check(c, "advance");
}

int ps3d_gpu_advance_host(ps3d_gpu_ctx *c, double *svor, double *t, ps3d_gpu_diag *diag)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!svor || !t) return PS3D_ERR_INVALID_ARG;
    if (c->cfg.buoyancy) return fail(c, PS3D_ERR_INVALID_ARG, "advance_host: the state of a buoyancy context includes sbuoy");
    const Dims &d = c->d;
    const size_t bytes = (size_t)3 * d.ncol * (d.nz + 1) * sizeof(double);
    // Page-locked host memory is read and written by the re-pitching
    // kernels themselves over the host link (zero copy); other host memory
    // goes through one linear copy each way into a staging array in host
    // layout (the RK accumulator svorf, free outside a step).
    double *mapped = nullptr;
    {
        cudaPointerAttributes pa;
        if (cudaPointerGetAttributes(&pa, svor) == cudaSuccess && pa.type == cudaMemoryTypeHost) {
            void *dp = nullptr;
            if (cudaHostGetDevicePointer(&dp, svor, 0) == cudaSuccess) mapped = static_cast<double *>(dp);
        }
        cudaGetLastError();
    }
    double *stage = mapped ? mapped : c->svorf;
    if (mapped && !c->fp64) {
        // mixed form, page-locked state: the host state is read over the
        // link into the staging array svorf and compared with the device
        // state on a second stream while the first right-hand side runs
        // from the device state; advance waits for the check before the
        // stage updates and evaluates the right-hand side again from the
        // host state if it differs (resolve_state_check)
        cudaEventRecord(c->ev_chk0, c->st);
        cudaStreamWaitEvent(c->st_chk, c->ev_chk0, 0);
        cudaMemsetAsync(c->flag_chk, 0, sizeof(int), c->st_chk);
        if (op_unpack_check(d, c->st_chk, mapped, c->svor, c->svorf, 3, c->flag_chk)) {
            cudaEventRecord(c->ev_chk, c->st_chk);
            c->pending_check = true;
            c->launches += 1;
            rc = ps3d_gpu_advance(c, t, 1, diag);
            if (c->pending_check) {  // the step stopped before adapt took the check
                cudaEventSynchronize(c->ev_chk);
                c->pending_check = false;
            }
            if (rc) return rc;
            op_pack_cols(d, c->st, c->svor, mapped, 3);
            c->launches += 1;
            return sync_check(c, "advance_host");
        }
    }
    if (!mapped) cudaMemcpyAsync(stage, svor, bytes, cudaMemcpyHostToDevice, c->st);
    cudaMemsetAsync(c->flag, 0, sizeof(int), c->st);
    op_unpack_cols(d, c->st, stage, c->svor, 3, c->flag);
    c->launches += 1;
    if (!c->fp64) {
        // a state bitwise equal to the device's (the previous step's result)
        // is already solenoidal; any other state is projected in FP64 first
        int changed = 0;
        cudaMemcpyAsync(&changed, c->flag, sizeof(int), cudaMemcpyDeviceToHost, c->st);
        rc = sync_check(c, "advance_host");
        if (rc) return rc;
        if (changed) project_state_mixed(c);
    }
    rc = ps3d_gpu_advance(c, t, 1, diag);
    if (rc) return rc;
    op_pack_cols(d, c->st, c->svor, stage, 3);
    c->launches += 1;
    if (!mapped) cudaMemcpyAsync(svor, stage, bytes, cudaMemcpyDeviceToHost, c->st);
    return sync_check(c, "advance_host");
}

int ps3d_gpu_calc_vorticity_mean(ps3d_gpu_ctx *c, double out[2])
{
    int rc = enter(c);
    if (rc) return rc;
    op_mean_fix(c->d, c->st, c->svor, c->dstsum, c->fnzi, c->ini, c->savg, 0);
    c->launches += 1;
    cudaMemcpyAsync(out, c->savg, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->st);
    return sync_check(c, "calc_vorticity_mean");
}

int ps3d_gpu_adjust_vorticity_mean(ps3d_gpu_ctx *c)
{
    int rc = enter(c);
    if (rc) return rc;
    op_mean_fix(c->d, c->st, c->svor, c->dstsum, c->fnzi, c->ini, nullptr, 1, c->svor32);
    c->launches += 1;
    return sync_check(c, "adjust_vorticity_mean");
}

int ps3d_gpu_energy_series(ps3d_gpu_ctx *c, double *ke, double *en, double *hel)
{
    int rc = enter(c);
    if (rc) return rc;
    double r1[RED1_N];
    rc = DISPATCH(c, energy, c, r1);
    if (rc) return rc;
    if (ke) *ke = 0.5 * r1[2] * c->ncelli;
    if (en) *en = 0.5 * r1[1] * c->ncelli;
    if (hel) *hel = r1[3] * c->ncelli;
    return PS3D_OK;
}

int ps3d_gpu_field_op(ps3d_gpu_ctx *c, int op, const double *in, double *out)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!in || !out) return PS3D_ERR_INVALID_ARG;
    return DISPATCH(c, field_op, c, op, in, out);
}

int ps3d_gpu_time_advance(ps3d_gpu_ctx *c, double *t, int nsteps, double *ms)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!t || !ms || nsteps < 0) return PS3D_ERR_INVALID_ARG;
    if (!c->diffusion_ready) return fail(c, PS3D_ERR_NOT_READY, "advance before init_diffusion");
    rc = sync_check(c, "time_advance");
    if (rc) return rc;
    cudaEventRecord(c->ev0, c->st);
    for (int s = 0; s < nsteps; ++s) {
        rc = DISPATCH(c, advance, c, t, nullptr);
        if (rc) return rc;
    }
    cudaEventRecord(c->ev1, c->st);
    rc = sync_check(c, "time_advance");
    if (rc) return rc;
    float f = 0.0f;
    cudaEventElapsedTime(&f, c->ev0, c->ev1);
    *ms = (double)f;
    return PS3D_OK;
}

int ps3d_gpu_advance_graph(ps3d_gpu_ctx *c, double *t, int nsteps, ps3d_gpu_diag *diag, double *ms)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!t || nsteps < 0) return PS3D_ERR_INVALID_ARG;
    rc = graph_prepare(c, *t);
    if (rc) return rc;
    cudaEventRecord(c->ev0, c->st);
    rc = graph_launch(c, nsteps);
    if (rc) return rc;
    cudaEventRecord(c->ev1, c->st);
    rc = graph_finish(c, t, diag);
    if (ms) {
        float f = 0.0f;
        cudaEventElapsedTime(&f, c->ev0, c->ev1);
        *ms = (double)f;
    }
    return rc;
}

int ps3d_gpu_batch_advance(ps3d_gpu_ctx *const *ctx, int n, double *t, int nsteps, double *ms)
{
    if (!ctx || !t || n <= 0 || nsteps < 0) return PS3D_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i) {
        if (!ctx[i] || ctx[i]->cfg.device != ctx[0]->cfg.device) return PS3D_ERR_INVALID_ARG;
        for (int j = 0; j < i; ++j)
            if (ctx[j] == ctx[i]) return fail(ctx[0], PS3D_ERR_INVALID_ARG, "batch: a context appears twice");
    }
    int rc = enter(ctx[0]);
    if (rc) return rc;
    for (int i = 0; i < n; ++i) {
        rc = graph_upload(ctx[i], t[i]);
        if (rc) return rc;
    }
    ps3d_gpu_ctx *c0 = ctx[0];
    if (!c0->batch || !c0->batch->same(ctx, n)) {
        delete c0->batch;
        c0->batch = new BatchPlan();
        c0->batch->runs.assign(ctx, ctx + n);
        for (int i = 0; i < n; ++i) c0->batch->serials.push_back(ctx[i]->serial);
        rc = batch_capture(c0->batch);
        if (rc) {
            delete c0->batch;
            c0->batch = nullptr;
            return rc;
        }
    }
    cudaStream_t s0 = c0->st;
    cudaEventRecord(c0->ev0, s0);
    for (int s = 0; s < nsteps && !rc; ++s)
        if (cudaGraphLaunch(c0->batch->exec, s0) != cudaSuccess) rc = check(c0, "batch launch");
    cudaEventRecord(c0->ev1, s0);
    c0->launches += c0->batch->kernels * nsteps;
    int rf = PS3D_OK;
    for (int i = 0; i < n; ++i) {
        // the runs' streams joined s0 inside the graph
        if (i > 0) cudaStreamWaitEvent(ctx[i]->st, c0->ev1, 0);
        const int r = graph_finish(ctx[i], &t[i], nullptr);
        if (r && !rf) rf = r;
    }
    if (ms) {
        float f = 0.0f;
        cudaEventElapsedTime(&f, c0->ev0, c0->ev1);
        *ms = (double)f;
    }
    return rc ? rc : rf;
}

int ps3d_gpu_tuning(ps3d_gpu_ctx *c, int shape[4], double ms[12])
{
    int rc = enter(c);
    if (rc) return rc;
    if (!shape || !ms) return PS3D_ERR_INVALID_ARG;
    for (int p = 0; p < 4; ++p) {
        shape[p] = c->d.line_shape[p];
        for (int w = 0; w < 3; ++w) ms[3 * p + w] = c->tune_ms[p][w];
    }
    return PS3D_OK;
}

int ps3d_gpu_set_tuning(ps3d_gpu_ctx *c, const int shape[4])
{
    int rc = enter(c);
    if (rc) return rc;
    if (!shape) return PS3D_ERR_INVALID_ARG;
    for (int p = 0; p < 4; ++p) {
        const int n = (p & 1) ? c->d.nx : c->d.ny;
        if (shape[p] < -1 || (shape[p] >= 0 && !lines32_has_shape(n, shape[p]))) return PS3D_ERR_INVALID_ARG;
    }
    if (c->graph) {  // a captured step holds the old shapes
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
    }
    for (int p = 0; p < 4; ++p) c->d.line_shape[p] = (signed char)shape[p];
    return PS3D_OK;
}

int ps3d_gpu_derived_fields(ps3d_gpu_ctx *c, double *pres, double *delta)
{
    int rc = enter(c);
    if (rc) return rc;
    return DISPATCH(c, derived_fields, c, pres, delta);
}

int ps3d_gpu_ke_spectrum(ps3d_gpu_ctx *c, int nmax, double *spec, int *nbins, double *dk)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!spec || !nbins || !dk || nmax < 1) return PS3D_ERR_INVALID_ARG;
    return DISPATCH(c, ke_spectrum, c, nmax, spec, nbins, dk);
}

int ps3d_gpu_host_alloc(size_t bytes, void **ptr)
{
    if (!ptr || bytes == 0) return PS3D_ERR_INVALID_ARG;
    *ptr = nullptr;
    if (cudaHostAlloc(ptr, bytes, cudaHostAllocPortable) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return PS3D_ERR_OUT_OF_MEMORY;
    }
    return PS3D_OK;
}

int ps3d_gpu_host_free(void *ptr)
{
    if (ptr && cudaFreeHost(ptr) != cudaSuccess) {
        cudaGetLastError();
        return PS3D_ERR_CUDA;
    }
    return PS3D_OK;
}

int ps3d_gpu_probe(ps3d_gpu_ctx *c, int kind)
{
    int rc = enter(c);
    if (rc) return rc;
    if (kind < PROBE_OFF || kind > PROBE_PRODUCTS) return PS3D_ERR_INVALID_ARG;
    rc = sync_check(c, "probe");
    if (rc) return rc;
    if (kind != PROBE_OFF && !c->probe.ev) {
        c->probe.ev = new cudaEvent_t[2 * Probe::MAXP];
        for (int i = 0; i < 2 * Probe::MAXP; ++i) cudaEventCreate(&c->probe.ev[i]);
    }
    c->probe.kind = kind;
    c->probe.used = 0;
    c->probe.launches = 0;
    c->probe.bytes = 0.0;
    return check(c, "probe");
}

int ps3d_gpu_probe_result(ps3d_gpu_ctx *c, double *total_ms, long long *launches, double *bytes)
{
    int rc = enter(c);
    if (rc) return rc;
    rc = sync_check(c, "probe_result");
    if (rc) return rc;
    double ms = 0.0;
    for (int i = 0; i + 1 < c->probe.used; i += 2) {
        float f = 0.0f;
        cudaEventElapsedTime(&f, c->probe.ev[i], c->probe.ev[i + 1]);
        ms += (double)f;
    }
    if (total_ms) *total_ms = ms;
    if (launches) *launches = c->probe.launches;
    if (bytes) *bytes = c->probe.bytes;
    return PS3D_OK;
}

int ps3d_gpu_synchronize(ps3d_gpu_ctx *c)
{
    int rc = enter(c);
    if (rc) return rc;
    return sync_check(c, "synchronize");
}

}  // extern "C"

// ------------------------------------------------------------ checkpoint
// Raw-binary checkpoint of everything a run carries from one step to the
// next.  Stored: the prognostic state svor (FP64, and in the mixed form its
// FP32 copy), the buoyancy state sbuoy (likewise), the rolling-mean rings of
// adapt with their indices, fill flags and running means, the initial mean
// vorticity, the viscosities vvisc / bvisc, the hyperdiffusion tables vhdis
// / bhdis, N^2 and the model time.  Not stored, because every step rebuilds
// them before use: vdiss / bdiss and the integrating factors epq, emq, epq2,
// emq2 (set_diffusion and the stepper's factor kernel recompute them from
// vhdis / bhdis, dt and the prefactor), and the grid tables of context
// creation (wavenumbers, filters, harmonic functions).  Restored
// without re-projection, a run continues bitwise (no result depends on the
// leftover content of padding rows: the line transforms read them as zero).
// The reference restarts
// from the physical vorticity of a NetCDF field file (utils.f90:102-116);
// its rolling means start afresh, so its restarts are not bit-continuous.

namespace {

struct CkptHeader {
    char magic[8];
    int32_t version, nx, ny, nz, precision, buoyancy, nnu, roll_len, rollb_len, diffusion_ready;
    int32_t roll_inew, roll_iold, roll_filled, rollb_inew, rollb_iold, rollb_filled;
    double t, lower[3], extent[3], ini_vor_mean[2], vvisc, bvisc, bfsq, roll_sma, rollb_sma;
};
constexpr char CKPT_MAGIC[8] = {'P', 'S', '3', 'D', 'G', 'P', 'U', 'S'};
constexpr int32_t CKPT_VERSION = 1;

// raw FP32 fields between device (P-pitched) and host ((nz+1)-pitched)
int f32_transfer(ps3d_gpu_ctx *c, float *dev, float *host, int ncomp, bool to_host)
{
    const Dims &d = c->d;
    const size_t hp = (size_t)(d.nz + 1) * sizeof(float);
    for (int k = 0; k < ncomp; ++k) {
        float *dk = dev + (size_t)k * d.nfield;
        float *hk = host + (size_t)k * (d.nz + 1) * d.ncol;
        const cudaError_t e =
            to_host ? cudaMemcpy2DAsync(hk, hp, dk, d.P * sizeof(float), hp, d.ncol, cudaMemcpyDeviceToHost, c->st)
                    : cudaMemcpy2DAsync(dk, d.P * sizeof(float), hk, hp, hp, d.ncol, cudaMemcpyHostToDevice, c->st);
        if (e != cudaSuccess) return check(c, "checkpoint transfer");
    }
    return sync_check(c, "checkpoint transfer");
}

struct File {
    FILE *f = nullptr;
    ~File()
    {
        if (f) fclose(f);
    }
};

}  // namespace

extern "C" {

int ps3d_gpu_save_state(ps3d_gpu_ctx *c, const char *path, double t)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!path) return PS3D_ERR_INVALID_ARG;
    const Dims &d = c->d;
    const size_t n1 = (size_t)(d.nz + 1) * d.ncol;
    CkptHeader h{};
    memcpy(h.magic, CKPT_MAGIC, 8);
    h.version = CKPT_VERSION;
    h.nx = d.nx;
    h.ny = d.ny;
    h.nz = d.nz;
    h.precision = c->cfg.precision;
    h.buoyancy = c->cfg.buoyancy ? 1 : 0;
    h.nnu = c->cfg.nnu;
    h.roll_len = (int32_t)c->roll.hist.size();
    h.rollb_len = (int32_t)c->roll_b.hist.size();
    h.diffusion_ready = c->diffusion_ready ? 1 : 0;
    h.roll_inew = c->roll.inew;
    h.roll_iold = c->roll.iold;
    h.roll_filled = c->roll.filled ? 1 : 0;
    h.rollb_inew = c->roll_b.inew;
    h.rollb_iold = c->roll_b.iold;
    h.rollb_filled = c->roll_b.filled ? 1 : 0;
    h.t = t;
    for (int k = 0; k < 3; ++k) {
        h.lower[k] = c->cfg.lower[k];
        h.extent[k] = c->cfg.extent[k];
    }
    h.ini_vor_mean[0] = c->ini_vor_mean[0];
    h.ini_vor_mean[1] = c->ini_vor_mean[1];
    h.vvisc = c->vvisc;
    h.bvisc = c->bvisc;
    h.bfsq = c->bfsq;
    h.roll_sma = c->roll.sma;
    h.rollb_sma = c->roll_b.sma;
    std::vector<double> vh(d.ncol, 0.0), bh(c->cfg.buoyancy ? d.ncol : 0, 0.0), sv(3 * n1), sb(c->cfg.buoyancy ? n1 : 0);
    std::vector<float> sv32(c->fp64 ? 0 : 3 * n1), sb32((!c->fp64 && c->cfg.buoyancy) ? n1 : 0);
    cudaMemcpyAsync(vh.data(), c->vhdis, d.ncol * sizeof(double), cudaMemcpyDeviceToHost, c->st);
    if (c->cfg.buoyancy) cudaMemcpyAsync(bh.data(), c->bhdis, d.ncol * sizeof(double), cudaMemcpyDeviceToHost, c->st);
    rc = download(c, c->svor, true, 3, sv.data());
    if (!rc && c->cfg.buoyancy) rc = download(c, c->sbuoy, true, 1, sb.data());
    if (!rc && !c->fp64) rc = f32_transfer(c, c->svor32, sv32.data(), 3, true);
    if (!rc && !c->fp64 && c->cfg.buoyancy) rc = f32_transfer(c, c->sbuoy32, sb32.data(), 1, true);
    if (!rc) rc = sync_check(c, "save_state");
    if (rc) return rc;
    File fh;
    fh.f = fopen(path, "wb");
    if (!fh.f) return fail(c, PS3D_ERR_INVALID_ARG, std::string("save_state: cannot open ") + path);
    bool ok = fwrite(&h, sizeof(h), 1, fh.f) == 1;
    auto put = [&](const void *p, size_t bytes) {
        if (ok && bytes) ok = fwrite(p, 1, bytes, fh.f) == bytes;
    };
    put(c->roll.hist.data(), c->roll.hist.size() * sizeof(double));
    put(c->roll_b.hist.data(), c->roll_b.hist.size() * sizeof(double));
    put(vh.data(), vh.size() * sizeof(double));
    put(bh.data(), bh.size() * sizeof(double));
    put(sv.data(), sv.size() * sizeof(double));
    put(sb.data(), sb.size() * sizeof(double));
    put(sv32.data(), sv32.size() * sizeof(float));
    put(sb32.data(), sb32.size() * sizeof(float));
    if (!ok) return fail(c, PS3D_ERR_INVALID_ARG, std::string("save_state: write failed for ") + path);
    return PS3D_OK;
}

int ps3d_gpu_load_state(ps3d_gpu_ctx *c, const char *path, double *t)
{
    int rc = enter(c);
    if (rc) return rc;
    if (!path || !t) return PS3D_ERR_INVALID_ARG;
    const Dims &d = c->d;
    const size_t n1 = (size_t)(d.nz + 1) * d.ncol;
    File fh;
    fh.f = fopen(path, "rb");
    if (!fh.f) return fail(c, PS3D_ERR_INVALID_ARG, std::string("load_state: cannot open ") + path);
    CkptHeader h{};
    if (fread(&h, sizeof(h), 1, fh.f) != 1 || memcmp(h.magic, CKPT_MAGIC, 8) != 0 || h.version != CKPT_VERSION)
        return fail(c, PS3D_ERR_INVALID_ARG, "load_state: not a checkpoint of this library version");
    bool same_box = true;
    for (int k = 0; k < 3; ++k)
        same_box = same_box && h.lower[k] == c->cfg.lower[k] && h.extent[k] == c->cfg.extent[k];
    if (h.nx != d.nx || h.ny != d.ny || h.nz != d.nz || h.precision != c->cfg.precision ||
        h.buoyancy != (c->cfg.buoyancy ? 1 : 0) || h.nnu != c->cfg.nnu || !same_box ||
        h.roll_len != (int32_t)c->roll.hist.size() || h.rollb_len != (int32_t)c->roll_b.hist.size())
        return fail(c, PS3D_ERR_INVALID_ARG, "load_state: checkpoint of another grid, box, form or configuration");
    // the ring indices address hist[inew-1] and hist[iold-1] on the next step
    // (rolling_mean.f90:36-69): a file with an index outside 1..len is refused
    if (h.roll_inew < 1 || h.roll_inew > h.roll_len || h.roll_iold < 1 || h.roll_iold > h.roll_len ||
        h.rollb_inew < 1 || h.rollb_inew > h.rollb_len || h.rollb_iold < 1 || h.rollb_iold > h.rollb_len)
        return fail(c, PS3D_ERR_INVALID_ARG, "load_state: rolling-mean index outside its ring");
    std::vector<double> rh(h.roll_len), rbh(h.rollb_len), vh(d.ncol), bh(h.buoyancy ? d.ncol : 0), sv(3 * n1),
        sb(h.buoyancy ? n1 : 0);
    std::vector<float> sv32(c->fp64 ? 0 : 3 * n1), sb32((!c->fp64 && h.buoyancy) ? n1 : 0);
    bool ok = true;
    auto get = [&](void *p, size_t bytes) {
        if (ok && bytes) ok = fread(p, 1, bytes, fh.f) == bytes;
    };
    get(rh.data(), rh.size() * sizeof(double));
    get(rbh.data(), rbh.size() * sizeof(double));
    get(vh.data(), vh.size() * sizeof(double));
    get(bh.data(), bh.size() * sizeof(double));
    get(sv.data(), sv.size() * sizeof(double));
    get(sb.data(), sb.size() * sizeof(double));
    get(sv32.data(), sv32.size() * sizeof(float));
    get(sb32.data(), sb32.size() * sizeof(float));
    if (!ok) return fail(c, PS3D_ERR_INVALID_ARG, "load_state: truncated checkpoint");
    // the state as saved: no projection, the FP32 copies verbatim
    rc = upload(c, sv.data(), 3, c->svor, true);
    if (!rc && !c->fp64) rc = f32_transfer(c, c->svor32, sv32.data(), 3, false);
    if (!rc && h.buoyancy) rc = upload(c, sb.data(), 1, c->sbuoy, true);
    if (!rc && h.buoyancy && !c->fp64) rc = f32_transfer(c, c->sbuoy32, sb32.data(), 1, false);
    if (rc) return rc;
    cudaMemcpyAsync(c->vhdis, vh.data(), d.ncol * sizeof(double), cudaMemcpyHostToDevice, c->st);
    if (h.buoyancy) {
        cudaMemcpyAsync(c->bhdis, bh.data(), d.ncol * sizeof(double), cudaMemcpyHostToDevice, c->st);
        c->bfsq = h.bfsq;
        for (int iz = 0; iz <= d.nz; ++iz) c->h_bbarz[iz] = c->bfsq * (c->cfg.lower[2] + (double)iz * c->dx[2]);
        cudaMemcpyAsync(c->bprof, c->h_bbarz.data(), (d.nz + 1) * sizeof(double), cudaMemcpyHostToDevice, c->st);
    }
    c->vvisc = h.vvisc;
    c->bvisc = h.bvisc;
    c->diffusion_ready = h.diffusion_ready != 0;
    c->roll.hist = rh;
    c->roll.inew = h.roll_inew;
    c->roll.iold = h.roll_iold;
    c->roll.filled = h.roll_filled != 0;
    c->roll.sma = h.roll_sma;
    c->roll_b.hist = rbh;
    c->roll_b.inew = h.rollb_inew;
    c->roll_b.iold = h.rollb_iold;
    c->roll_b.filled = h.rollb_filled != 0;
    c->roll_b.sma = h.rollb_sma;
    c->closure_fresh = true;
    *t = h.t;
    rc = sync_check(c, "load_state");
    if (rc) return rc;
    return ps3d_gpu_set_ini_vor_mean(c, h.ini_vor_mean);
}

}  // extern "C"
