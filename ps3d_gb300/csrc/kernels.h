// Internal launcher declarations shared by the translation units of
// libps3d_gpu.so (not part of the public C ABI).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "common.cuh"

struct ps3d_closure;

namespace ps3d {

struct Dims {
    int nx, ny, nz;
    int P;                // padded column pitch (>= nz+1, multiple of 8)
    long long ncol;       // nx*ny
    long long nfield;     // P*ny*nx elements per scalar field
    // FP32 line-FFT block shape per pass, picked by the autotuner:
    // [0] forward y, [1] forward x, [2] inverse y, [3] inverse x;
    // -1 = the default shape of the line length
    signed char line_shape[4] = {-1, -1, -1, -1};
};

enum { COL_DST = 0, COL_DCT = 1, COL_DECOMP = 2, COL_COMBINE = 3 };

// Optional timing probe: brackets every launch of one kernel class with CUDA
// events on the launching stream (used by the benchmark to time the dominant
// kernel inside a real step).  kind: 0 off, 1 y lines, 2 x lines, 3 columns.
// PROBE_LINES brackets the line transforms of both directions
enum { PROBE_OFF = 0, PROBE_YLINES = 1, PROBE_XLINES = 2, PROBE_COLUMNS = 3, PROBE_LINES = 4, PROBE_PRODUCTS = 5 };
struct Probe {
    static constexpr int MAXP = 8192;
    int kind = PROBE_OFF;
    cudaEvent_t *ev = nullptr;  // 2*MAXP events
    int used = 0;
    long long launches = 0;
    double bytes = 0.0;         // algorithmic bytes of the bracketed launches
    bool match(int k) const
    {
        return k == kind || (kind == PROBE_LINES && (k == PROBE_YLINES || k == PROBE_XLINES));
    }
    void begin(int k, cudaStream_t st)
    {
        if (match(k) && ev && used + 2 <= 2 * MAXP) cudaEventRecord(ev[used++], st);
    }
    void end(int k, cudaStream_t st, double b)
    {
        if (match(k) && ev && (used & 1)) {
            cudaEventRecord(ev[used++], st);
            ++launches;
            bytes += b;
        }
    }
};

// transforms.cu
void transforms_init();
// horizontal transforms of nf consecutive fields (nfield apart), one launch
// per pass where the FP32 line kernels serve the length
template <typename T>
void xy_forward(const Dims &d, cudaStream_t st, const T *in, T *out, const typename cplx<T>::type *twx,
                const typename cplx<T>::type *twy, Probe *pr, int nf = 1);
template <typename T>
void x_forward(const Dims &d, cudaStream_t st, const T *in, T *out, const typename cplx<T>::type *twx, Probe *pr,
               int nf = 1);
template <typename T>
void x_inverse(const Dims &d, cudaStream_t st, const T *in, T *out, const typename cplx<T>::type *twx, Probe *pr,
               int nf = 1);
template <typename T>
void y_inverse(const Dims &d, cudaStream_t st, const T *in, T *out, const typename cplx<T>::type *twy, Probe *pr,
               int nf = 1);
template <typename T>
void xy_inverse(const Dims &d, cudaStream_t st, const T *in, T *out, const typename cplx<T>::type *twx,
                const typename cplx<T>::type *twy, Probe *pr, int nf = 1);
template <typename T>
void columns(const Dims &d, cudaStream_t st, int mode, const T *in, T *out, const T *phim,
             const T *phip, const typename cplx<T>::type *twz2, Probe *pr);
// FP32 bandwidth-tuned line FFTs (lines32.cu), n = 64..1024
bool lines32_supported(int n);
void lines32_init();
// shape: -1 default, 0 the default blocks (512 threads, two per SM, at
// n = 512), 1 256-thread blocks (three per SM, n = 512), 2 the TMA-fed
// persistent kernel (n = 128..512); a shape the length lacks runs the default
// zv = nz+1 valid z rows; rows zv..P-1 (padding) are read as zero
// nf fields per launch: field f at in + f fs_in, out + f fs_out
void launch_lines32(cudaStream_t st, const float *in, float *out, int n, int P, int zv, long long line_stride,
                    long long nbatch, long long batch_stride, bool inverse, const float2 *tw, int shape = -1,
                    int nf = 1, long long fs_in = 0, long long fs_out = 0);
// kernel shapes at line length n: 0 the default blocks, 1 256-thread blocks
// (n = 512), 2 the TMA-fed persistent kernel (n = 128, 256, 512)
bool lines32_has_shape(int n, int w);
int lines32_shapes(int n);  // how many of them n has
// a bounded wait of the TMA-fed kernel ran out since the last call (cleared)
// the forward y lines of the five products of vorticity_tendency (r, q,
// p, dq/dz, dp/dz; out holds them nfield apart) formed from the physical
// velocity and vorticity inside the line kernel (ny = 64..1024)
bool lines32_prod_supported(int ny);
void lines32_prod_y(cudaStream_t st, const float *vel, const float *vor, float *out, const Dims &d, double dzi,
                    const float2 *twy, Probe *pr);
int lines32_error();
// FP32 half-length warp z transforms (colz.cu), nz = 64..1024
bool colz_supported(int nz);
void colz_init();
// 1 (and cleared) when a column kernel's bounded wait for a staged copy ran
// out, or a launch was refused for breaking the kernels' 16-byte layout rules
int colz_error();
template <typename TIN>
void columns_z(const Dims &d, cudaStream_t st, int mode, const TIN *in, float *out, const double *k2l2, float dz,
               float Lz, const float2 *twn, const float *sinz, const float *cosz, Probe *pr);
// fused column kernels of the mixed form (colz.cu): the vertical velocity
// of vor2vel (w and dw/dz from ds), and the decomposition of the third
// tendency component together with the z part of its solenoidal projection
// (out = decompose(f), es = decompose(central_diffz(f)); out may be f)
void columns_w(const Dims &d, cudaStream_t st, const float *ds, float *w, float *es, const double *k2l2,
               const double *k2l2i, float dz, float Lz, const float2 *twn, const float *sinz, const float *cosz,
               Probe *pr);
// w and dw/dz of vor2vel with the w source ds formed inside the column
// kernels from the state components A, B (nz = 64..512)
bool columns_w_src_supported(int nz);
void columns_w_src(const Dims &d, cudaStream_t st, const float *A, const float *B, float *w, float *es,
                   const double *k2l2, const double *k2l2i, const double *cx, const double *cy, float dz, float Lz,
                   const float2 *twn, const float *sinz, const float *cosz, Probe *pr);
// the tail of the mixed source: tendency components from the transformed
// products, decomposed, and es (three column kernels); corr (nullable): an
// attached closure's semi-spectral correction, three fields nfield apart,
// added to the components before their decomposition
void columns_src(const Dims &d, cudaStream_t st, const float *r, const float *q, const float *p, const float *gq,
                 const float *gp, float *s1, float *s2, float *s3, float *es, const double *k2l2, const double *cx,
                 const double *cy, float dz, float Lz, const float2 *twn, const float *sinz, Probe *pr,
                 const float *corr = nullptr);
void columns_dec2(const Dims &d, cudaStream_t st, const float *f, float *out, float *es, const double *k2l2,
                  float dz, float Lz, const float2 *twn, const float *sinz, Probe *pr);
// FP32 warp-per-column-pair transforms (columns32.cu), nz = 32..512
bool col32_supported(int nz);
void columns32_init();
template <typename TIN>
void columns32(const Dims &d, cudaStream_t st, int mode, const TIN *in, float *out, const double *k2l2, float dz,
               float Lz, const float2 *twL, Probe *pr);
// column transform of an FP64 input field into a T field (mixed form)
template <typename T, typename TIN>
void columns_in(const Dims &d, cudaStream_t st, int mode, const TIN *in, T *out, const T *phim,
                const T *phip, const typename cplx<T>::type *twz2, Probe *pr);

// Spectral-horizontal derivative operators.  For a spectral index k along
// x (or y) the reference's diffx/diffy (sta3dfft.f90:304-377, with the
// single-rank reverse_x/y of mpi_reverse.f90) reduce to
//    (D f)(k) = c[k] * f(src[k]),   src[k] = (n - k) mod n,
// with c[k] = -hrk(2k) for 1 <= k < n/2, +hrk(2(n-k)) for k > n/2 and
// c[0] = c[n/2] = 0.
struct Deriv {
    const double *cx;  // nx
    const double *cy;  // ny
};

struct Tables {
    // per (ky,kx) column (ny*nx, FP64)
    const double *k2l2i, *filt0, *vhdis, *epq, *emq, *epq2, *emq2, *vdiss;
    // per kz (nz+1, FP64)
    const double *fz;       // vertical Hou-Li / 2/3 factor, fz[0] = fz[nz] = 1
    const double *rkz, *rkzi, *gamtop, *gambot, *dstsum, *dctcos;
};

// ops.cu : elementwise / stencil kernels (T = transient field type, S = state)
template <typename T> void op_diff(const Dims &d, cudaStream_t st, const Deriv &D, int axis, const T *in, T *out);
template <typename T> void op_diffz(const Dims &d, cudaStream_t st, double dzi, const T *in, T *out);
template <typename T, typename S>
void op_v2v_ds(const Dims &d, cudaStream_t st, const Deriv &D, const S *A, const S *B, T *ds);
template <typename T, typename S>
void op_v2v_project(const Dims &d, cudaStream_t st, const Deriv &D, const double *k2l2i, const T *es,
                    const T *ds, S *A, S *B);
template <typename T, typename S>
void op_v2v_wsrc(const Dims &d, cudaStream_t st, const Deriv &D, const S *A, const S *B, T *ds);
template <typename T>
void op_v2v_wprep(const Dims &d, cudaStream_t st, const T *ds, const T *thetam, const T *thetap,
                  const T *dthetam, const T *dthetap, const T *green, const double *rkz, T *bs, T *es,
                  T *dsg, T *as);
template <typename T>
void op_v2v_wfinish(const Dims &d, cudaStream_t st, const T *dsg, const T *bs, const T *as, T *w, T *es);
template <typename S>
void op_v2v_meanflow(const Dims &d, cudaStream_t st, const S *A, const S *B, const Tables &tb, double *ubar,
                     double *vbar);
template <typename T>
void op_v2v_uv(const Dims &d, cudaStream_t st, const Deriv &D, const double *k2l2i, const T *es, const T *cs,
               const double *ubar, const double *vbar, T *u, T *v);
template <typename T>
void op_add_const(const Dims &d, cudaStream_t st, T *f, double c);
template <typename T>
void op_products(const Dims &d, cudaStream_t st, const T *vel, const T *vor, T *r, T *q, T *p);
// products and the z derivatives gq = dq/dz, gp = dp/dz in one pass
template <typename T>
void op_products_dz(const Dims &d, cudaStream_t st, double dzi, const T *vel, const T *vor, T *r, T *q, T *p,
                    T *gq, T *gp);
template <typename T>
void op_svorts(const Dims &d, cudaStream_t st, const Deriv &D, const T *r, const T *q, const T *p,
               const T *gq, const T *gp, T *s1, T *s2, T *s3);
template <typename T>
void op_strain_fields(const Dims &d, cudaStream_t st, const Deriv &D, const T *svel, T *g5);
template <typename T, typename S>
void op_convert(const Dims &d, cudaStream_t st, const S *in, T *out, long long n);
template <typename T, typename S>
void op_add(const Dims &d, cudaStream_t st, S *acc, const T *add, long long n);

// steppers
template <typename T>
void op_rk4_sub1(const Dims &d, cudaStream_t st, double *q, double *qdi, double *qdf, T *sqs,
                 const double *filt0, const double *emq, double dt2, double dt6);
template <typename T>
void op_rk4_sub23(const Dims &d, cudaStream_t st, double *q, const double *qdi, double *qdf, const T *sqs,
                  const double *epq, const double *emq, double c1, double dt3);
template <typename T>
void op_rk4_sub4(const Dims &d, cudaStream_t st, double *q, const double *qdf, const T *sqs,
                 const double *epq, const double *emq, double dt6);
void op_rk4_factors(const Dims &d, cudaStream_t st, const double *vdiss, const double *filt0, double *epq,
                    double *emq, double *epq2, double *emq2);
template <typename T>
void op_cn2_init(const Dims &d, cudaStream_t st, double *vortsm, const double *svor, const T *svorts,
                 double dt2, int ncomp = 3);
template <typename T>
void op_cn2_update(const Dims &d, cudaStream_t st, double *svor, const double *vortsm, const T *svorts,
                   const double *filt0, const double *fz, const double *vdiss, double dt2, int ncomp = 3);
void op_mean_fix(const Dims &d, cudaStream_t st, double *svor, const double *dstsum, double fnzi,
                 const double *ini, double *savg_out, int apply, float *svor32 = nullptr);
// mixed-form stage updates (FP64 state, FP32 source, state copy and
// accumulated source increments acc)
// (dtp: the step's dt in device memory; full: the third stage's full-step factor)
void op_rk4m_sub1(const Dims &d, cudaStream_t st, double *q, double *qdi, float *acc, const float *sqs, float *q32,
                  const double *filt0, const double *emq, const double *dtp);
void op_rk4m_sub23(const Dims &d, cudaStream_t st, double *q, const double *qdi, float *acc, const float *sqs,
                   float *q32, const double *epq, const double *emq, const double *dtp, bool full);
void op_rk4m_sub4(const Dims &d, cudaStream_t st, double *q, const double *qdi, const float *acc, const float *sqs,
                  float *q32, const double *epq, const double *emq, const double *dtp);
void op_narrow(cudaStream_t st, const double *in, float *out, long long n);
// mixed form, impl-diff-rk4: the solenoidal projection of the tendency
// (S: the three decomposed components; es: decompose(diffz(S3))), the
// filter and substep sub (1..4) of the integrating-factor RK4 in one pass;
// fp, fm: the substep's column factors (1: filt0, emq; 2: epq, emq;
// 3: epq, emq2; 4: epq2, emq2).  The FP64 state q is rewritten by substep 4
// only; mf receives the (0,0) column of each stage state (components 1, 2)
void op_stage_orbit(const Dims &d, cudaStream_t st, int sub, const Deriv &D, const double *k2l2i, const float *S,
                    const float *es, double *q, float *acc, float *q32, double *mf, const double *fp,
                    const double *fm, const double *dtp);
// one run of a batch for op_batch_stage: the arguments of op_stage_orbit,
// the column factors of the four substeps, and the number of the run's
// first work item (one item per partner orbit, runs numbered in order)
struct StageRun {
    Dims d;
    Deriv D;
    const double *k2l2i;
    const float *S, *es;
    double *q;
    float *acc, *q32;
    double *mf;
    const double *fp[4], *fm[4];
    const double *dtp;
    long long item0;
};
// the stage update of every run of a batch in one persistent launch
// (runs: device array of nruns entries; nitems: all runs' orbits)
void op_batch_stage(cudaStream_t st, int sub, const StageRun *runs, int nruns, long long nitems, int blocks);
int batch_stage_blocks();
// derived fields (pressure right-hand side, table product, horizontal divergence)
template <typename T> void op_pressure_rhs(const Dims &d, cudaStream_t st, const T *g5, const T *vor, T *out);
template <typename T> void op_mul_field(const Dims &d, cudaStream_t st, const T *tab, T *f);
template <typename T> void op_hdiv(const Dims &d, cudaStream_t st, const Deriv &D, const T *svel, T *out);
// kinetic-energy shell binning of the spectral velocity f (3 components)
template <typename T>
void op_spec_bins(const Dims &d, cudaStream_t st, const double *rkx, const double *rky, const double *rkz,
                  const T *f, double dki, int kmax, double *bins, unsigned long long *cnt);
// host-layout (nz+1)-pitched FP64 columns <-> device P-pitched columns
void op_unpack_cols(const Dims &d, cudaStream_t st, const double *src, double *dst, int ncomp, int *changed);
void op_pack_cols(const Dims &d, cudaStream_t st, const double *src, double *dst, int ncomp);
// host-layout state -> staging array in the device layout, compared bitwise
// with cmp (*changed raised on a difference); a small persistent grid meant
// to run beside other kernels.  false (nothing launched): src not 16-byte
// aligned.
bool op_unpack_check(const Dims &d, cudaStream_t st, const double *src, const double *cmp, double *dst, int ncomp,
                     int *changed);

// reductions (adapt, energy series); results are FP64 partials per block
struct RedOut {
    double *part;     // scratch partials
    double *result;   // final values
};
template <typename T>
void red_pass1(const Dims &d, cudaStream_t st, const T *vel, const T *vor, double *part, double *result);
template <typename T>
// vortrms from the pass-1 results on the device when res1 is given:
// sqrt(res1[1] / ncell)
void red_pass2(const Dims &d, cudaStream_t st, const T *vor, const T *g5, double vortrms, double *part,
               double *result, int *flag, const double *res1 = nullptr, double ncell = 1.0);
int red_nblocks(const Dims &d);

// buoyancy.cu: diffz pieces, flux products, tendency assembly, maximum
// buoyancy frequency and buoyancy diagnostics
template <typename T>
void op_dphi_tables(const Dims &d, cudaStream_t st, const double *k2l2, const double *zm, const double *zp, double Lz,
                    T *dphim, T *dphip);
template <typename T> void op_dz_sine(const Dims &d, cudaStream_t st, const double *rkz, const T *fs, T *as);
template <typename T>
void op_dz_join(const Dims &d, cudaStream_t st, const T *fs, const T *dphim, const T *dphip, const T *as, T *ds);
template <typename T> void op_bflux(const Dims &d, cudaStream_t st, const T *vel, const T *b, T *f);
template <typename T>
void op_btend(const Dims &d, cudaStream_t st, const Deriv &D, const T *fu, const T *fv, const T *wsemi, const T *zs,
              double bfsq, T *out);
template <typename T> void op_addf(const Dims &d, cudaStream_t st, T *f, const T *g);
void op_sub_zprof(const Dims &d, cudaStream_t st, double *f, const double *prof);
template <typename T>
void op_pres_buoy_rhs(const Dims &d, cudaStream_t st, const T *b, const T *zeta, double dzi, double fz, T *out);
template <typename T>
void op_pres_buoy_bc(const Dims &d, cudaStream_t st, const T *sb, const double *k2l2i, const T *dphim, const T *dphip,
                     T *rs);
template <typename T>
void op_bgrad_max(const Dims &d, cudaStream_t st, const T *bx, const T *by, const T *b, double dzi, double bfsq,
                  unsigned long long *out);
long long bdiag_blocks(const Dims &d);
template <typename T>
void op_bdiag(const Dims &d, cudaStream_t st, const T *b, const T *bx, const T *by, const T *vor, double dzi,
              double bfsq, double *part, double *out);
constexpr int RED1_N = 12;  // values of pass 1
constexpr int RED2_N = 5;   // values of pass 2

// tables
template <typename T>
void op_hyperbolic_tables(const Dims &d, cudaStream_t st, const double *k2l2, const double *k2l2i,
                          const double *rkz, const double *zm, const double *zp, double Lz, T *phim, T *phip,
                          T *thetam, T *thetap, T *dthetam, T *dthetap, T *green);

// closure.cu: the learned sub-grid closure's side of a context
int closure_attach(ps3d_closure *cl, const void *owner, int nx, int ny, int nz, int device, std::string *err);
void closure_detach(ps3d_closure *cl, const void *owner);
// physical correction out[c] (c*ostride + iz + pitch*col) from the physical
// vor and vel of a run; no host synchronisation
template <typename T>
int closure_apply(ps3d_closure *cl, cudaStream_t st, const T *vor, const T *vel, long long cstride, int pitch, T *out,
                  long long ostride, int flags);
constexpr int CLOSURE_LAUNCHES = 9;

size_t lines_smem_bytes(int n, bool fp64);
size_t columns_smem_bytes(int nz, bool fp64);

}  // namespace ps3d
