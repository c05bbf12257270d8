/*
 * pwd_gb300.h -- C ABI of the GB300 plane-wave-destruction library
 * (libpwd_gb300.so).
 *
 * Drop-in boundary for pyseistr's structural hot path.  Each entry point
 * replaces one low-level CPython entry of the reference and takes the same
 * arguments with the same meaning, but on device memory:
 *
 *   - arrays are float32, column-major (Fortran order, time axis n1
 *     fastest: i = i1 + n1*(i2 + n2*i3)), exactly as the reference's Python
 *     wrappers flatten them before calling C;
 *   - every pointer is a device pointer the caller allocated; the entry
 *     points allocate no device memory, their scratch is the caller's
 *     `workspace` of at least the size the matching *_workspace_size()
 *     returns (256-byte aligned) -- except pwd_dip_static, whose scratch is
 *     a fixed device array of the library (below);
 *   - work is enqueued on `stream` (NULL = legacy default stream) and the
 *     call returns without synchronising; results are ready once the
 *     stream has been synchronised (pwd_sint2d, pwd_sint3d,
 *     pwd_soint2d_prec and pwd_soint2d_prec_batch read values back and
 *     synchronise `stream` before they return);
 *   - results depend only on the arguments: calls on different streams
 *     with different workspaces may run concurrently.  The library's own
 *     process-wide state is limited to pwd_dip_static's scratch array
 *     (shared by every call of that entry) and the launch counter and
 *     optional timing profiler of pwd_launch_count / pwd_profile_*
 *     (bookkeeping guarded by a mutex, never read by the compute path);
 *   - errors are returned as pwd_status codes (the reference prints and
 *     returns NULL, which surfaces as SystemError).
 *
 * The plain path reproduces the reference's float arithmetic operation by
 * operation, including its quirks (effective divne/CG eps = 1, eps forced
 * to 0.01 in the 3-D filters, the triangle-weighted 2-D mean).
 */
#ifndef PWD_GB300_H
#define PWD_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *pwd_stream_t; /* same object as cudaStream_t */

typedef enum {
  PWD_OK = 0,
  PWD_EINVAL = 1,      /* bad size or parameter (reference: "Dimension mismatch") */
  PWD_EWORKSPACE = 2,  /* workspace missing, too small or misaligned */
  PWD_ECUDA = 3,       /* a CUDA launch or runtime call failed */
  PWD_ENOTSUP = 4      /* valid for the reference but not built here (order > 4) */
} pwd_status;

/* Library version as 10000*major + 100*minor + patch. */
int pwd_version(void);
/* Static description of a status code. */
const char *pwd_status_string(int status);

/* ------------------------------------------------------------------------
 * Local slope by plane-wave destruction.
 * Replaces dipc, pyseistr/src/dip_cfuns.c:1694-1989 (called by dip2dc,
 * dip2d.py:115, and dip3dc, dip3d.py:59).
 *   data     [n1*n2*n3]; mask [n1*n2*n3] or NULL (the reference appends the
 *            mask to the data array and sets hasmask=1)
 *   dip_out  n3 == 1: [n1*n2] inline slope;
 *            n3 > 1 : [2*n1*n2*n3] inline slope, then crossline slope
 *   niter    nonlinear (Gauss-Newton) iterations; liter: CG iterations of
 *            the shaping division; order: PWD accuracy order (1..4);
 *   rect     triangle smoothing radius per axis (1 = no smoothing)
 * eps_dv / eps_cg / tol_cg of the reference are accepted by the Python
 * layer and ignored there, as the reference C ignores them.
 */
size_t pwd_dip_workspace_size(int n1, int n2, int n3, int order, const int rect[3],
                              int has_mask);
int pwd_dip(const float *data, const float *mask, float *dip_out, int n1, int n2, int n3,
            int niter, int liter, int order, const int rect[3], void *workspace,
            size_t workspace_bytes, pwd_stream_t stream);

/* ------------------------------------------------------------------------
 * Slope estimation that allocates nothing.  No counterpart in the reference
 * (which has no GPU code): it serves callers that cannot allocate device
 * memory when they estimate slopes -- a plugin inside a host application
 * that owns the CUDA context and its memory budget, or a real-time loop
 * that must not call cudaMalloc (which can synchronise the device) after
 * start-up.  Same arguments and results as pwd_dip, without the workspace:
 * the scratch is a file-scope device array of pwd_dip_static_capacity()
 * bytes (64 MiB), resident on every GPU that loads the library until the
 * process exits.  Sections whose pwd_dip_workspace_size() exceeds it are
 * rejected with PWD_EWORKSPACE before any work is enqueued.
 *   - Every call looks up the array's device address in the current
 *     context (cudaGetSymbolAddress, with the device current; it allocates
 *     nothing), so a cudaDeviceReset between calls is harmless.  The first
 *     call in a context loads the library's device code there (lazy module
 *     loading, the CUDA default), which commits the array's memory and can
 *     stall like an allocation: make one warm-up call at start-up, before
 *     any stream capture on the device (or set CUDA_MODULE_LOADING=EAGER,
 *     which commits the array when the library is loaded).
 *   - Every call uses the same array; each call initialises the parts it
 *     reads, but calls that overlap on the GPU (different streams, or
 *     threads without ordering) race on it and give wrong results.
 */
size_t pwd_dip_static_capacity(void);
int pwd_dip_static(const float *data, const float *mask, float *dip_out, int n1, int n2, int n3,
                   int niter, int liter, int order, const int rect[3], pwd_stream_t stream);

/* ------------------------------------------------------------------------
 * Batched slope estimation over many independent sections of uneven size
 * (the patch / DAS-window workflows), in one fixed launch sequence: every
 * kernel covers all sections.  Same results as one pwd_dip call per
 * section.  The section table is read from host memory during the call.
 * No single reference entry point: it replaces a loop of dipc calls
 * (dip_cfuns.c:1694) over the sections.
 */
typedef struct {
  long offset;     /* element offset of the section in data (and mask) */
  long out_offset; /* element offset of its slopes in dip_out (2n for 3-D) */
  int n1, n2, n3;
} pwd_section;

size_t pwd_dip_batch_workspace_size(const pwd_section *sections, int nsec, int order,
                                    const int rect[3], int has_mask);
int pwd_dip_batch(const float *data, const float *mask, float *dip_out,
                  const pwd_section *sections, int nsec, int niter, int liter, int order,
                  const int rect[3], void *workspace, size_t workspace_bytes,
                  pwd_stream_t stream);

/* pwd_dip_batch / pwd_dip_batch_mixed split in two for CUDA graphs.
 * pwd_dip_batch_prepare copies the section table into the workspace (a
 * host-to-device copy on stream; the workspace must be sized for the mode
 * and mask); pwd_dip_batch_run then enqueues only kernels and memsets, so
 * a stream capture of it can be replayed for new contents of data (and
 * mask) at the same addresses.  mixed selects the mixed mode.  No
 * reference counterpart (the reference has no GPU launch sequence).
 */
int pwd_dip_batch_prepare(const pwd_section *sections, int nsec, int order, const int rect[3],
                          int has_mask, int mixed, void *workspace, size_t workspace_bytes,
                          pwd_stream_t stream);
int pwd_dip_batch_run(const float *data, const float *mask, float *dip_out,
                      const pwd_section *sections, int nsec, int niter, int liter, int order,
                      const int rect[3], int mixed, void *workspace, size_t workspace_bytes,
                      pwd_stream_t stream);

/* Mixed mode of pwd_dip_batch (same arguments).  Not bit-faithful: the
 * filter taps are evaluated in FP32, the triangle smoothing of the shaping
 * CG is applied as the equivalent direct convolution (triangle weights
 * (nb-|k|)/nb^2 on the half-sample-mirrored line) fused with the CG vector
 * updates, and the dot products stay in FP64 as in the plain path.  The
 * slopes agree with an FP64 evaluation of the reference algorithm to about
 * the accuracy of the plain FP32 path.  No reference counterpart: it is an
 * alternative arithmetic for the same dipc computation.  Its tile copies
 * wait at most 50 ms each; a section whose copy did not complete in time
 * (a fault of the device, not of the input) gets NaN slopes.
 */
size_t pwd_dip_batch_mixed_workspace_size(const pwd_section *sections, int nsec, int order,
                                          const int rect[3], int has_mask);
int pwd_dip_batch_mixed(const float *data, const float *mask, float *dip_out,
                        const pwd_section *sections, int nsec, int niter, int liter, int order,
                        const int rect[3], void *workspace, size_t workspace_bytes,
                        pwd_stream_t stream);

/* ------------------------------------------------------------------------
 * 2-D structure-oriented mean, slice by slice over n3.
 * Replaces csomean2d, pyseistr/src/sof_cfuns.c:1433-1531 (somean2dc,
 * somean2d.py:36): triangle-weighted spray mean normalised by the spray of
 * ones; adj != 0 applies the adjoint.
 */
size_t pwd_somean2d_workspace_size(int n1, int n2, int n3, int ns, int order);
int pwd_somean2d(const float *data, const float *dip, float *out, int n1, int n2, int n3,
                 int ns, int order, int adj, float eps, void *workspace,
                 size_t workspace_bytes, pwd_stream_t stream);

/* ------------------------------------------------------------------------
 * 2-D structure-oriented median filter, slice by slice over n3.
 * Replaces csomf2d, pyseistr/src/sof_cfuns.c:1534-1678 (somf2dc,
 * somf2d.py:60).  nmf: median window (somf2dc passes 2*ns+1);
 * option 1 = median filter, otherwise space-varying median (svmf).
 */
size_t pwd_somf2d_workspace_size(int n1, int n2, int n3, int ns, int nmf, int option,
                                 int order);
int pwd_somf2d(const float *data, const float *dip, float *out, int n1, int n2, int n3, int ns,
               int nmf, int option, int order, float eps, void *workspace,
               size_t workspace_bytes, pwd_stream_t stream);

/* ------------------------------------------------------------------------
 * Batched 2-D structure-oriented filters over many sections of uneven size
 * in one launch sequence: filter 1 = mean (csomean2d adj=0), 2 = adjoint
 * mean (adj=1), 3 = median (csomf2d with nmf, option).  data and dip share
 * the sections' offsets; the filtered output of section k is written at
 * sections[k].out_offset.  Same results as one call per section; replaces
 * a loop of csomean2d / csomf2d calls (sof_cfuns.c:1433, :1534).
 */
size_t pwd_sofilter2d_batch_workspace_size(const pwd_section *sections, int nsec, int ns,
                                           int order, int filter, int nmf, int option);
int pwd_sofilter2d_batch(const float *data, const float *dip, float *out,
                         const pwd_section *sections, int nsec, int ns, int order, int filter,
                         int nmf, int option, float eps, void *workspace,
                         size_t workspace_bytes, pwd_stream_t stream);

/* ------------------------------------------------------------------------
 * 3-D structure-oriented mean over the (2*r1+1)*(2*r2+1) spray.
 * Replaces csomean3d, pyseistr/src/sof3d_cfuns.c:1355-1551 (somean3dc,
 * somean3d.py:36).  eps is accepted and replaced by 0.01 as the reference.
 */
size_t pwd_somean3d_workspace_size(int n1, int n2, int n3, int r1, int r2, int order);
int pwd_somean3d(const float *data, const float *dip_inline, const float *dip_xline,
                 float *out, int n1, int n2, int n3, int r1, int r2, int order, float eps,
                 void *workspace, size_t workspace_bytes, pwd_stream_t stream);

/* ------------------------------------------------------------------------
 * 3-D structure-oriented median filter.
 * Replaces csomf3d, pyseistr/src/sof3d_cfuns.c:1554-1753 (somf3dc,
 * somf3d.py:54).  nmf: median length (somf3dc passes 2*r1*r2+1), taken
 * over raster-ordered spray slots centred on the centre slot.
 */
size_t pwd_somf3d_workspace_size(int n1, int n2, int n3, int r1, int r2, int nmf, int option,
                                 int order);
int pwd_somf3d(const float *data, const float *dip_inline, const float *dip_xline, float *out,
               int n1, int n2, int n3, int r1, int r2, int nmf, int option, int order,
               float eps, void *workspace, size_t workspace_bytes, pwd_stream_t stream);

/* ------------------------------------------------------------------------
 * Median along the spray axis of given sprayed panels, centre row only.
 * Replaces mf / svmf (pyseistr/src/sof_cfuns.c:1294-1332, :1334-1431, with
 * mf_init/svmf_init axis=2 ifbound=1) as csomf2d/csomf3d apply them:
 *   panels [ntr][np][n1] (each source trace's np sprayed traces),
 *   out    [ntr][n1]     row (np-1)/2 of the filtered panel.
 */
size_t pwd_panel_median_workspace_size(int n1, int np, long ntr, int nmf, int option);
int pwd_panel_median(const float *panels, float *out, int n1, int np, long ntr, int nmf,
                     int option, void *workspace, size_t workspace_bytes, pwd_stream_t stream);

/* ------------------------------------------------------------------------
 * 3-D structure-oriented interpolation (PWD-regularised CG).
 * Replaces csoint3d, pyseistr/src/soint3d_cfuns.c:2405-2507 (soint3dc,
 * soint3d.py:65).  known = (mask != 0) if hasmask == 1, else (data != 0);
 * var > 0 adds the reference's seeded MT19937/Box-Muller noise to the
 * zero data of the PWD residual.
 */
size_t pwd_soint3d_workspace_size(int n1, int n2, int n3, int order);
int pwd_soint3d(const float *data, const float *mask, const float *dip_inline,
                const float *dip_xline, float *out, int n1, int n2, int n3, int order, int nj1,
                int nj2, int niter, int drift, int seed, int hasmask, float var,
                void *workspace, size_t workspace_bytes, pwd_stream_t stream);

/* ------------------------------------------------------------------------
 * 2-D interpolation preconditioned by plane-wave integration.
 * Replaces the prec = 1 branches of csoint2d, pyseistr/src/soint2d_cfuns.c:
 * 2354-2398 (soint2dc(..., prec=1), soint2d.py:92): ps_solver_prec
 * (:1704) on M P p = d with ps_cgstep, P = predict_lop (:1537) along dip1,
 * or predict2_lop (:1597) chaining dip1 and dip2 when twoplane; out = P p.
 * known = (mask != 0) if hasmask == 1, else (data != 0).  n1 >= 2.  The
 * call synchronises `stream` (it reads back a completion flag) and returns
 * PWD_ECUDA if a trace's factor copy did not complete in time.
 */
size_t pwd_soint2d_prec_workspace_size(int n1, int n2, int order, int twoplane);
int pwd_soint2d_prec(const float *data, const float *mask, const float *dip1, const float *dip2,
                     float *out, int n1, int n2, int order, int niter, int hasmask,
                     int twoplane, void *workspace, size_t workspace_bytes,
                     pwd_stream_t stream);
/* Many 2-D sections of uneven size (n3 = 1) at once, one CTA each: a loop
 * of csoint2d(prec = 1) calls.  sections[k].offset places section k in
 * data, mask and out, sections[k].out_offset its slopes in dip1 (and dip2)
 * as pwd_dip_batch writes them; at most 65535 sections.  Every section
 * gets the results of its own pwd_soint2d_prec call.  Synchronises
 * `stream`. */
size_t pwd_soint2d_prec_batch_workspace_size(const pwd_section *sections, int nsec, int order,
                                             int twoplane);
int pwd_soint2d_prec_batch(const float *data, const float *mask, const float *dip1,
                           const float *dip2, float *out, const pwd_section *sections,
                           int nsec, int order, int niter, int hasmask, int twoplane,
                           void *workspace, size_t workspace_bytes, pwd_stream_t stream);

/* Many patches of uneven size in one launch sequence (the batched
 * interpolation workflow): a loop of csoint3d calls over patches without
 * noise (var = 0).  sections[k].offset places patch k in data, mask and
 * out; sections[k].out_offset places its slopes in dips as pwd_dip_batch
 * writes them (inline n, then crossline n), so the two calls chain.  Every
 * patch gets the results of its own pwd_soint3d call.
 */
size_t pwd_soint3d_batch_workspace_size(const pwd_section *sections, int nsec, int order);
int pwd_soint3d_batch(const float *data, const float *mask, const float *dips, float *out,
                      const pwd_section *sections, int nsec, int order, int nj1, int nj2,
                      int niter, int drift, int hasmask, void *workspace,
                      size_t workspace_bytes, pwd_stream_t stream);

/* ------------------------------------------------------------------------
 * Launch accounting and kernel timing (no counterpart in the reference,
 * which has no GPU code).  Kernel families:
 */
enum {
  PWD_FAM_PWD = 0,      /* PWD residual / derivative / line-search trials  */
  PWD_FAM_CG = 1,       /* shaping-CG vector updates and reductions        */
  PWD_FAM_TRIANGLE = 2, /* triangle-smoothing line sweeps                  */
  PWD_FAM_SPRAY = 3,    /* plane-wave spray chains / trees                 */
  PWD_FAM_FILTER = 4,   /* spray mean / median reductions                  */
  PWD_FAM_SOINT = 5,    /* interpolation operator and CG                   */
  PWD_FAM_OTHER = 6,
  PWD_NFAM = 7
};
/* ---- Patching (pyseistr/patch.py mode 1) --------------------------------
 * An n1 x n2 x n3 column-major array (n3 = l3 = s3 = 1 for patch2d) cut into
 * l1 x l2 x l3 windows at strides s1, s2, s3, each axis zero-padded at its
 * end to n + s - mod(n - l, s) when mod(n - l, s) != 0; patch id runs over
 * the first axis's window starts outermost; x = [npatch][l1 l2 l3], each
 * patch column-major (the packed-section layout of the batched entries).
 * Replace patch2d (patch.py:2), patch3d (:86), patch2d_inv (:208) and
 * patch3d_inv (:307).  The inverse adds the patches covering each sample in
 * FP64 in patch order, divides by their count (NaN where none covers it)
 * and rounds to float.  Device pointers; no workspace. */
/* Number of patches, 0 for invalid sizes, for more than 2^31 - 1 patch
 * elements, or for an axis with no window (a window longer than the axis
 * when the stride divides the excess: the reference's loops then make no
 * patch at all). */
size_t pwd_patch_count(int n1, int n2, int n3, int l1, int l2, int l3, int s1, int s2, int s3);
int pwd_patch(const float *a, float *x, int n1, int n2, int n3, int l1, int l2, int l3, int s1,
              int s2, int s3, pwd_stream_t stream);
int pwd_patch_inv(const float *x, float *a, int n1, int n2, int n3, int l1, int l2, int l3,
                  int s1, int s2, int s3, pwd_stream_t stream);

/* ---- Band-pass (pyseistr/bp.py bandpassc, src/bp_cfuns.c cbp) ------------
 * Replaces cbp (bp_cfuns.c:524, argument tuple "Oiiifffiiii" less the verb
 * flag): Butterworth low-cut (flo) and high-cut (fhi) filters along each of
 * the n2*n3 column-major traces of length n1; flo, fhi in Hz with d1 the
 * sampling interval (a negative cut-off is taken as already in cycles per
 * sample); flo <= 1e-4 cycles per sample skips the low cut and fhi >=
 * 0.5 - 1e-4 the high cut; nplo, nphi poles (at least 1, halved when
 * phase = 0); phase 0 runs each filter forward then backward (zero phase),
 * 1 forward only.  Results are bit-identical to cbp's.  `out` may equal
 * `in`.  Device pointers; no workspace. */
int pwd_bandpass(const float *in, float *out, int n1, int n2, int n3, float d1, float flo,
                 float fhi, int nplo, int nphi, int phase, pwd_stream_t stream);

/* ---- Radon coherence (pyseistr/das.py cohc, src/coh_cfuns.c cohc_fb) ----
 * Replaces cohc_fb (coh_cfuns.c:415, argument tuple "OOOiiiifii" less the
 * verb flag) with coh_init2 (:158) and coh (:181).  Model [nv][nt], data
 * [nh][nt], column-major; v[nv] curve parameters, h[nh] offsets; typ 1
 * linear (t = itau dt + h v), 2 parabolic (itau dt + h^2 v / hmax / hmax),
 * 3 hyperbolic (sqrt(tau^2 + (h / v)^2)), any other value linear; sample
 * floor(t / dt) + 1 for 0 <= it <= nt, as flat indices into the data (it = nt
 * is the next trace's first sample).  forw = 1: `in` is the model, `out` the
 * data (the terms added in the reference's order; the past-the-end sample
 * of the last trace dropped).  forw = -1: `in` is the data, `out` the model
 * num^2 / (nh den + 1e-16) of the stack num and energy den along each
 * curve.  Where a curve reaches past the end of the data (sample nt of the
 * last trace) the reference reads whatever follows its array (undefined:
 * NaN or garbage); that sample reads as 0 here.  Results are bit-identical
 * to cohc_fb's on every other sample.  `hmax` is the parabolic normaliser that the reference keeps
 * in a file-scope static across calls (updated from h by coh_init2); the
 * caller keeps and passes it.  Curves whose sample index is NaN or at least
 * 2e9 in magnitude add nothing (the reference converts them to int with an
 * undefined result; the Python layer refuses them).  Device pointers; no
 * workspace; `out` must not overlap `in`. */
int pwd_coherence(const float *in, const float *v, const float *h, int typ, int nt, int nv,
                  int nh, float dt, int forw, float hmax, float *out, pwd_stream_t stream);
/* nwin windows of the same sizes stacked one after another in `in` and
 * `out` (the windows of a DAS record, as the detection loop of
 * demos/test_pyseistr_das_massive.py:190-203 calls cohc on each), in one
 * launch: the same results as one pwd_coherence call per window (each
 * window's past-the-end sample reads as 0).  No single reference entry: it
 * replaces that loop of cohc_fb calls. */
int pwd_coherence_batch(const float *in, const float *v, const float *h, int typ, int nt, int nv,
                        int nh, int nwin, float dt, int forw, float hmax, float *out,
                        pwd_stream_t stream);

/* ---- Plane-wave painting (pyseistr/rgt.py pwpaintc, rgt; src/paint_cfuns.c
 * cpaint2d) ---------------------------------------------------------------
 * Replaces cpaint2d (paint_cfuns.c:1861, argument tuple "OOiiiifi" less the
 * verb flag): the seed trace seed[n1] placed at trace i0 of out[n2][n1] and
 * carried to both ends by the PWD prediction step along the slopes
 * dip[n2][n1] (leftwards along the slope of the trace reached, rightwards
 * along the slope of the trace before it), with accuracy order 1..4 and
 * regularisation eps (squared, as predict_init takes it).  Results are
 * bit-identical to cpaint2d's.  Serial along the traces: one thread per
 * side of the section.  Device pointers; the workspace holds both threads'
 * band arrays (pwd_paint2d_workspace_size bytes, 0 for n1 < 4 or an order
 * outside 1..4); i0 outside [0, n2) is PWD_EINVAL (the reference writes out
 * of bounds). */
size_t pwd_paint2d_workspace_size(int n1, int order);
int pwd_paint2d(const float *dip, const float *seed, float *out, int n1, int n2, int order,
                int i0, float eps, void *workspace, size_t workspace_bytes, pwd_stream_t stream);
/* nsec sections of one size stacked one after another (dip and out at s n1
 * n2, seed at s n1), each painted from its own seed trace at trace i0, in
 * one launch: the same results as one pwd_paint2d call per section.  No
 * single reference entry: it replaces a loop of cpaint2d calls. */
size_t pwd_paint2d_batch_workspace_size(int n1, int nsec, int order);
int pwd_paint2d_batch(const float *dip, const float *seed, float *out, int n1, int n2, int nsec,
                      int order, int i0, float eps, void *workspace, size_t workspace_bytes,
                      pwd_stream_t stream);

/* ---- Sparse-data interpolation (pyseistr/sint.py sint2dc, src/soint2d_cfuns.c
 * csint2d) ------------------------------------------------------------------
 * Replaces csint2d (soint2d_cfuns.c:2421, argument tuple "OOOiiiiiif" less
 * the verb flag): the (n1, n2) section din with known samples where mask
 * != 0, interpolated by niter shaping-regularised CG iterations whose
 * shaping is the plane-wave smoothing of csomean2d (spray radius ns,
 * accuracy order 1..4, regularisation eps) along the slopes dip, started
 * from din, with lambda = sqrt(known / n) and the reference's stopping
 * test.  Every float operation is the reference's; the dot products are
 * FP64 sums in another order, so a scalar can differ in its last double
 * bits.  The call synchronises `stream` twice per iteration (the CG's
 * decisions are taken on the host).  Device pointers; workspace of
 * pwd_sint2d_workspace_size bytes (0 for invalid sizes); out must not
 * overlap the inputs. */
size_t pwd_sint2d_workspace_size(int n1, int n2, int ns, int order);
int pwd_sint2d(const float *din, const float *dip, const float *mask, float *out, int n1, int n2,
               int niter, int ns, int order, float eps, void *workspace, size_t workspace_bytes,
               pwd_stream_t stream);
/* Replaces csint3d (soint3d_cfuns.c:2510, tuple "OOOOiiiiiiiiif" less the
 * verb flag): the same CG on an (n1, n2, n3) cube whose shaping smooths every
 * (n1, n2) slice along the inline slopes dipi (radius ns1, order order1),
 * then every (n1, n3) section along the crossline slopes dipx (ns2, order2),
 * the adjoint in reverse (pwsmooth3_lop, :2157-2300).  Same arithmetic,
 * synchronisation and workspace rules as pwd_sint2d. */
size_t pwd_sint3d_workspace_size(int n1, int n2, int n3, int ns1, int ns2, int order1,
                                 int order2);
int pwd_sint3d(const float *din, const float *dipi, const float *dipx, const float *mask,
               float *out, int n1, int n2, int n3, int niter, int ns1, int ns2, int order1,
               int order2, float eps, void *workspace, size_t workspace_bytes,
               pwd_stream_t stream);

/* ---- FK dip filter (pyseistr/fk.py fkdip) ---------------------------------
 * Replaces fkdip (fk.py:2, numpy in the reference): the part of the
 * (n1, n2) section d inside the cone of half-width w nk columns around k = 0
 * of its FK spectrum, back in time and space, as float64 out[n2][n1] (the
 * reference returns float64).  The FFTs are zero-padded to nf =
 * nextpow2(n1) and nk = nextpow2(n2); the time and space FFTs run in the
 * input's precision (complex64 for pwd_fkdip, complex128 for pwd_fkdip_f64,
 * as numpy keeps the input's precision), the mask promotes to complex128 and
 * the inverse FFTs run in complex128.  Not bit-identical to numpy's FFTs:
 * about 1e-7 relative for float input, 1e-15 for double.  w = 0 is
 * PWD_EINVAL (the reference divides by zero).  Device pointers; workspace
 * of pwd_fkdip_workspace_size bytes (f64: the double entry's; 0 for
 * invalid sizes).  Each call uploads its twiddle tables from host memory
 * with cudaMemcpyAsync, so it cannot be captured into a CUDA graph. */
size_t pwd_fkdip_workspace_size(int n1, int n2, int f64);
int pwd_fkdip(const float *d, double *out, int n1, int n2, double w, void *workspace,
              size_t workspace_bytes, pwd_stream_t stream);
int pwd_fkdip_f64(const double *d, double *out, int n1, int n2, double w, void *workspace,
                  size_t workspace_bytes, pwd_stream_t stream);

/* Number of kernels the library has launched since it was loaded. */
unsigned long long pwd_launch_count(void);
/* Start recording a CUDA event pair around every launch (process-wide; for
 * benchmarks, not for concurrent use from several threads). */
void pwd_profile_start(void);
/* Stop recording; synchronises the recorded events and writes, per family,
 * the summed kernel time in ms and the number of launches (arrays of
 * `nfam` entries).  Returns the number of launches recorded. */
int pwd_profile_stop(double *ms, int *launches, int nfam);
/* FP32 FMA throughput probe (no reference counterpart): `blocks` x
 * `threads` threads each run 8 independent FMA chains of `iters` steps
 * (16 flops per step) and write one float to out[thread]; time it with
 * CUDA events to measure the FP32 CUDA-core peak. */
int pwd_fp32_fma_probe(float *out, int blocks, int threads, int iters, pwd_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* PWD_GB300_H */
