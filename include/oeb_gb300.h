/*
 * oeb_gb300.h -- C ABI of the GB300 (sm_103a) open-earth-benchmarks stencils.
 *
 * Every entry point takes field descriptors laid out exactly like the reference's
 * strided Storage<T,R> (include/util.h:24-31): {allocatedPtr, alignedPtr, offset,
 * sizes[R], strides[R]}, with element (i,j,k) at
 *     aligned[offset + strides[2]*i + strides[1]*j + strides[0]*k]
 * (include/util.h:82-94), i.e. i is the unit-stride axis and sizes/strides are
 * stored k-first.  The descriptor of the reference's allocateStorage
 * (include/util.h:126-141) is accepted as is; any row/plane padding is also
 * accepted as long as strides[2] == 1.
 *
 * The reference reads the interior extents from the globals domain_size and
 * domain_height (src/<k>.cpp:4-5); here they are the explicit oeb_domain
 * {nx, ny, nz}, which also allows nx != ny.
 *
 * Device entry points (oeb_<k>_f64 / _f32) take DEVICE pointers and are
 * asynchronous on the given cudaStream_t (passed as void*, NULL = legacy default
 * stream).  Host entry points (oeb_<k>_f64_host) take HOST pointers -- run on them
 * in place where the device can address host memory, else staged through device
 * memory -- and return after the outputs are in host memory.  No entry point writes the scratch fields of the reference signatures
 * (lap/flx/fly, T_sqr_s, uatupos..., ppgk..., wk, du, dv, fxx, al, ...): they are
 * not parameters of this ABI.  Cells outside each output's written box are left
 * untouched, as in the reference.
 *
 * All functions return an oeb_status; nothing aborts the process.
 */
#ifndef OEB_GB300_H
#define OEB_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define OEB_API __attribute__((visibility("default")))
#else
#define OEB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum oeb_status {
  OEB_OK = 0,
  OEB_ERR_NULL = 1,        /* a required descriptor or pointer is NULL                     */
  OEB_ERR_DOMAIN = 2,      /* nx, ny or nz < 1, or the domain exceeds the 2^31 index limit */
  OEB_ERR_LAYOUT = 3,      /* strides[2] != 1, strides not nested, or the 3-D fields of     */
                           /* one call do not share strides                                 */
  OEB_ERR_HALO = 4,        /* a field's halo is smaller than the kernel's reach             */
  OEB_ERR_ALIGNMENT = 5,   /* a pointer is not aligned to its element size                  */
  OEB_ERR_CUDA = 6,        /* a CUDA runtime call failed; see oeb_last_cuda_error()         */
  OEB_ERR_ALLOC = 7,       /* device or pinned allocation failed                            */
  OEB_ERR_ALIAS = 8,       /* an output field overlaps an input field                       */
  OEB_ERR_UNSUPPORTED = 9, /* unknown kernel or variant                                      */
  OEB_ERR_TIMEOUT = 10,    /* a bounded device-side wait gave up                             */
  OEB_ERR_TOO_LARGE = 11,  /* a request exceeds a documented fixed capacity                  */
  OEB_ERR_ARGUMENT = 12    /* a scalar argument is out of its documented range               */
} oeb_status;

typedef struct oeb_memref3d_f64 {
  double* allocated;
  double* aligned;
  int64_t offset;
  int64_t sizes[3];   /* {k extent, j extent, i extent} incl. halo (util.h:129-131) */
  int64_t strides[3]; /* {k stride, j stride, i stride == 1}    (util.h:133-135) */
} oeb_memref3d_f64;

typedef struct oeb_memref1d_f64 {
  double* allocated;
  double* aligned;
  int64_t offset;
  int64_t sizes[1];
  int64_t strides[1];
} oeb_memref1d_f64;

typedef struct oeb_memref3d_f32 {
  float* allocated;
  float* aligned;
  int64_t offset;
  int64_t sizes[3];
  int64_t strides[3];
} oeb_memref3d_f32;

typedef struct oeb_memref1d_f32 {
  float* allocated;
  float* aligned;
  int64_t offset;
  int64_t sizes[1];
  int64_t strides[1];
} oeb_memref1d_f32;

/* Interior extents: nx = ny = domain_size and nz = domain_height in the reference. */
typedef struct oeb_domain {
  int64_t nx;
  int64_t ny;
  int64_t nz;
} oeb_domain;

/* ------------------------------------------------------------------------- */
/* Library information and errors                                             */
/* ------------------------------------------------------------------------- */

/* ABI version: major * 10000 + minor * 100 + patch. */
OEB_API int oeb_abi_version(void);
/* Static, NUL-terminated description of a status code. */
OEB_API const char* oeb_status_string(int status);
/* Text of the last CUDA error seen by this thread ("" if none). */
OEB_API const char* oeb_last_cuda_error(void);
/* Number of kernel launches this library has issued (all threads) since load.  */
OEB_API uint64_t oeb_launch_count(void);
/* 1 if `p` points to device (or managed) memory, 0 if to host memory; used by the C++
 * drop-in headers to pick the device or the host-buffer entry point. */
OEB_API int oeb_is_device_pointer(const void* p);
/* Blocks until all work on `stream` has finished (NULL = legacy default stream). */
OEB_API oeb_status oeb_stream_synchronize(void* stream);
/* k-levels each CTA of the tiled stencils covers (1..1024), for every later call on every
 * thread; 0 (the default) restores each kernel's own choice.  A tuning knob: results do not
 * depend on it.  Batch plans record and tune their own. */
OEB_API oeb_status oeb_set_kblock(int kb);
/* Tile shape of the pointwise advection kernels (hadvuv, hadvuv5th and their adjoint terms),
 * for every later call on every thread: 0 (the default) 32 x 32 cells a CTA, 1 = 32 x 8,
 * 2 = 64 x 16.  OEB_ERR_ARGUMENT for any other value.  A tuning knob: results do not depend
 * on it.  Batch plans choose their own shapes (oeb_batch_autotune). */
OEB_API oeb_status oeb_set_tile_shape(int shape);
/* Fusion groupings of the chained step (no counterpart in the reference, which has no chained
 * step): a bit mask of stages that run as one kernel in every later oeb_chain_* call.
 * OEB_FUSE_HADV_UPDATE: hadvuv5th and the explicit update u2 = u1 + dt_adv * tendency in one
 * kernel (the advection writes u2, v2 directly), and in the adjoint step the hadvuv5th
 * gather and the update's transpose in one kernel; the default (faster in both precisions).
 * 0: separate kernels.  OEB_ERR_ARGUMENT for other bits.  A tuning knob: results do not
 * depend on it.  Batch plans choose their own grouping (created with 0; oeb_batch_autotune,
 * oeb_batch_set_fusion). */
/* 1 (the default): the FP32 adjoints of hdiffsmag, hadvuv, hadvuv5th, fastwavesuv, p_grad_c
 * and nh_p_grad run as one tiled launch that forms its terms (coefficients) in shared memory;
 * 0: as their multi-pass form, the terms in scratch.  No counterpart in the reference.  Results do not
 * depend on it (the same operations on the same operands); OEB_ERR_ARGUMENT for other
 * values. */
OEB_API oeb_status oeb_set_adjoint_tiles(int on);
#define OEB_FUSE_HADV_UPDATE 1
#define OEB_FUSE_ALL 1
OEB_API oeb_status oeb_set_fusion(int mask);
/* k-slabs of the host entry points' copy/compute/copy pipeline (1..8), for every later call;
 * 0 (the default) picks 8 for synchronous calls that move 8 MB or more, and 1 for smaller
 * and for asynchronous calls.  A tuning knob: results do not depend on it. */
OEB_API oeb_status oeb_set_host_slabs(int slabs);
/* 1 (the default): host entry points run the kernels on the host fields in place when the
 * device can address all of them (pageable memory on systems whose GPU uses the host page
 * tables, such as Grace-Blackwell; page-locked memory mapped at the same address elsewhere);
 * 0: always stage through device memory.  Results do not depend on it. */
OEB_API oeb_status oeb_set_host_direct(int enable);
/* 0 (the default): host entry points return once their outputs are in host memory.
 * 1: they return once their work is enqueued; the outputs are in host memory when `stream`
 * has completed (synchronise it), and the host fields must stay valid and unchanged until
 * then.  Asynchronous calls always stage through device memory, one slab a call, and
 * pipeline across calls on one device: a call's copy-in overlaps the previous calls'
 * compute and copy-out.  Host memory should be page-locked (pageable source memory makes
 * the driver's copies synchronous).  Results do not depend on it. */
OEB_API oeb_status oeb_set_host_async(int enable);

/* Self-check of the FP64 operations that the FP64 kernels run on the integer pipe: op 0
 * multiply, 1 divide, 2 add, 3 subtract, 4 square root of a.  `pairs` seeded random
 * operand pairs of distribution `mode` (0: any bit pattern; 1: magnitudes 2^-40..2^40;
 * 2: exponents within 60 of the normal range's ends; 3: short significands, which make
 * rounding ties; 4: significands near all-ones and near zero; 5: b times a small integer,
 * and b (for the square root: exact squares); 6: a and -a (1 + small), cancellation; 7: a
 * and a 2^-k with changed low bits, every alignment) are computed both ways on the current
 * device; `mismatches` receives how many results differ in any bit (NaNs compare equal),
 * `first` (4 words, may be NULL) the first differing a, b, FP64-instruction result and
 * integer-pipe result.  Synchronous. */
OEB_API oeb_status oeb_selftest_fp64(int op, int64_t pairs, uint64_t seed, int mode, uint64_t* mismatches,
                                     uint64_t* first);
/* No counterpart in the reference (a measurement of the GPU the FP64 stencils run on): the FP64
 * pipe's issue rate, as FP64 additions a second over every SM -- eight independent chains of
 * __dadd_rn a thread, eight CTAs of 256 threads an SM, the fastest of three timed launches
 * after a warm-up.  `adds_per_launch` (may be NULL) receives the additions of one launch.
 * Synchronous, on the legacy default stream. */
OEB_API oeb_status oeb_probe_fp64_add_rate(double* adds_per_second, double* adds_per_launch);
/* The rate of one FP64 operation on this GPU, measured the same way (no counterpart in the
 * reference): op 0 addition, 1 multiplication, 2 fused multiply-add, 3 division, 4 square
 * root (3 and 4: the compiler's IEEE-rounded instruction sequences), in operations a second,
 * and the operations one timed launch performs.  OEB_ERR_ARGUMENT for another op. */
OEB_API oeb_status oeb_probe_fp64_rate(int op, double* ops_per_second, double* ops_per_launch);
/* No counterpart in the reference (a measurement behind the stencils' design): i-neighbours
 * read through L1 against warp shuffles, FP32, on a 256 x 256 x 80 interior with a 3-cell
 * halo.  us[0..3] receive the average launch time (microseconds; the best of three runs of 60
 * back-to-back launches rotating over 12 input copies, more than the L2) of the 5-point
 * laplacian with loaded i-neighbours, the same with shuffled ones (lanes 0 and 31 load the
 * warp's outer cells), a 7-cell window along i loaded, and the same window shuffled.
 * mismatches[0..1] receive the cells where the two forms of the laplacian and of the window
 * differ in any bit (0 expected).  Allocates and frees about 330 MB; synchronous, on the
 * legacy default stream. */
OEB_API oeb_status oeb_probe_shuffle_neighbours(double* us, uint64_t* mismatches);

/* ------------------------------------------------------------------------- */
/* Device storage (the device twin of allocateStorage/freeStorage,           */
/* include/util.h:99-148).  The element layout is the reference's, with the  */
/* row pitch rounded up to pitch_multiple elements (1 = no padding).          */
/* ------------------------------------------------------------------------- */

OEB_API oeb_status oeb_storage3d_alloc_f64(int64_t nx, int64_t ny, int64_t nz, int64_t halo, int64_t pitch_multiple,
                                   oeb_memref3d_f64* out);
OEB_API oeb_status oeb_storage1d_alloc_f64(int64_t n, int64_t halo, oeb_memref1d_f64* out);
OEB_API oeb_status oeb_storage3d_alloc_f32(int64_t nx, int64_t ny, int64_t nz, int64_t halo, int64_t pitch_multiple,
                                   oeb_memref3d_f32* out);
OEB_API oeb_status oeb_storage1d_alloc_f32(int64_t n, int64_t halo, oeb_memref1d_f32* out);
/* Frees a descriptor returned by oeb_storage*_alloc_* and clears its pointers. */
OEB_API oeb_status oeb_storage_free(void* memref);
/* Whole-field transfers (the device side of include/util.h:99-148, which has no device
 * fields): oeb_upload* copies a host field to its device twin, oeb_download* back.  The
 * descriptors must have the same offset, sizes and strides.  Accepted pairs: a host field
 * made by the reference's allocateStorage (aligned = allocated + 32 - halo) or by any other
 * allocator of that layout, with a device field from oeb_storage*_alloc_* of the same sizes,
 * halo and pitch_multiple 1 (aligned = allocated), in either direction; the allocated
 * pointers take no part.  The elements from aligned[0] to the last one are copied, halo and
 * row padding included.  The copy uses cudaMemcpyDefault, so either side may be host memory
 * (pageable or pinned) or device memory.  Asynchronous on `stream`: synchronise it before
 * reading a downloaded field or changing an uploaded host field.  OEB_ERR_NULL,
 * OEB_ERR_LAYOUT, or OEB_ERR_ALIAS (the element ranges overlap) are returned before any CUDA
 * call. */
OEB_API oeb_status oeb_upload3d_f64(const oeb_memref3d_f64* dev, const oeb_memref3d_f64* host, void* stream);
OEB_API oeb_status oeb_download3d_f64(const oeb_memref3d_f64* host, const oeb_memref3d_f64* dev, void* stream);
OEB_API oeb_status oeb_upload1d_f64(const oeb_memref1d_f64* dev, const oeb_memref1d_f64* host, void* stream);
OEB_API oeb_status oeb_download1d_f64(const oeb_memref1d_f64* host, const oeb_memref1d_f64* dev, void* stream);
OEB_API oeb_status oeb_upload3d_f32(const oeb_memref3d_f32* dev, const oeb_memref3d_f32* host, void* stream);
OEB_API oeb_status oeb_download3d_f32(const oeb_memref3d_f32* host, const oeb_memref3d_f32* dev, void* stream);
OEB_API oeb_status oeb_upload1d_f32(const oeb_memref1d_f32* dev, const oeb_memref1d_f32* host, void* stream);
OEB_API oeb_status oeb_download1d_f32(const oeb_memref1d_f32* host, const oeb_memref1d_f32* dev, void* stream);
/* Bytes spanned by a descriptor: from allocated to one past the last element. */
OEB_API int64_t oeb_memref3d_span_bytes_f64(const oeb_memref3d_f64* m);
OEB_API int64_t oeb_memref3d_span_bytes_f32(const oeb_memref3d_f32* m);

/* ------------------------------------------------------------------------- */
/* FP64 forward stencils, device pointers, asynchronous on `stream`.          */
/* Argument order is the reference signature's with the scratch fields and    */
/* the globals made explicit.                                                 */
/* ------------------------------------------------------------------------- */

/* kernels/laplace.h:4 -- laplace(in, out) */
OEB_API oeb_status oeb_laplace_f64(const oeb_memref3d_f64* in, const oeb_memref3d_f64* out, const oeb_domain* dom,
                           void* stream);

/* kernels/hdiffsa.h:4-5 -- hdiffsa(out, in, mask, crlato, crlatu, lap, flx, fly) */
OEB_API oeb_status oeb_hdiffsa_f64(const oeb_memref3d_f64* out, const oeb_memref3d_f64* in, const oeb_memref3d_f64* mask,
                           const oeb_memref1d_f64* crlato, const oeb_memref1d_f64* crlatu, const oeb_domain* dom,
                           void* stream);

/* kernels/hdiffsmag.h:4-7 -- hdiffsmag(uout, vout, uin, vin, mask, crlavo, crlavu, crlato, crlatu,
 *                                      acrlat0, T_sqr_s, S_sqr_uv, eddlat, eddlon, tau_smag, weight_smag) */
OEB_API oeb_status oeb_hdiffsmag_f64(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                             const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                             const oeb_memref3d_f64* mask, const oeb_memref1d_f64* crlavo,
                             const oeb_memref1d_f64* crlavu, const oeb_memref1d_f64* crlato,
                             const oeb_memref1d_f64* crlatu, const oeb_memref1d_f64* acrlat0, double eddlat,
                             double eddlon, double tau_smag, double weight_smag, const oeb_domain* dom,
                             void* stream);

/* kernels/hadvuv.h:29-32 -- hadvuv(uout, vout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1,
 *                                  uatupos, vatupos, uatvpos, vatvpos, uavg, vavg, ures, vres, eddlat, eddlon) */
OEB_API oeb_status oeb_hadvuv_f64(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout, const oeb_memref3d_f64* uin,
                          const oeb_memref3d_f64* vin, const oeb_memref1d_f64* acrlat0,
                          const oeb_memref1d_f64* acrlat1, const oeb_memref1d_f64* tgrlatda0,
                          const oeb_memref1d_f64* tgrlatda1, double eddlat, double eddlon, const oeb_domain* dom,
                          void* stream);

/* kernels/hadvuv5th.h:41-44 -- hadvuv5th(same arguments as hadvuv) */
OEB_API oeb_status oeb_hadvuv5th_f64(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                             const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                             const oeb_memref1d_f64* acrlat0, const oeb_memref1d_f64* acrlat1,
                             const oeb_memref1d_f64* tgrlatda0, const oeb_memref1d_f64* tgrlatda1, double eddlat,
                             double eddlon, const oeb_domain* dom, void* stream);

/* kernels/fastwavesuv.h:4-7 -- fastwavesuv(uout, vout, uin, vin, utens, vtens, wgtfac, ppuv, hhl, rho, fx,
 *                                          ppgk, ppgc, ppgu, ppgv, edadlat, dt) */
OEB_API oeb_status oeb_fastwavesuv_f64(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                               const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                               const oeb_memref3d_f64* utens, const oeb_memref3d_f64* vtens,
                               const oeb_memref3d_f64* wgtfac, const oeb_memref3d_f64* ppuv,
                               const oeb_memref3d_f64* hhl, const oeb_memref3d_f64* rho, const oeb_memref1d_f64* fx,
                               double edadlat, double dt, const oeb_domain* dom, void* stream);

/* kernels/uvbke.h:4-5 -- uvbke(ub, vb, uc, vc, cosa, rsina); dt5 is the driver global (src/uvbke.cpp:11-12) */
OEB_API oeb_status oeb_uvbke_f64(const oeb_memref3d_f64* ub, const oeb_memref3d_f64* vb, const oeb_memref3d_f64* uc,
                         const oeb_memref3d_f64* vc, const oeb_memref3d_f64* cosa, const oeb_memref3d_f64* rsina,
                         double dt5, const oeb_domain* dom, void* stream);

/* kernels/nh_p_grad.h:4-6 -- nh_p_grad(uout, vout, uin, vin, rdx, rdy, gz, pp, pk3, wk1, wk, du, dv, dt) */
OEB_API oeb_status oeb_nh_p_grad_f64(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                             const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref3d_f64* rdx,
                             const oeb_memref3d_f64* rdy, const oeb_memref3d_f64* gz, const oeb_memref3d_f64* pp,
                             const oeb_memref3d_f64* pk3, const oeb_memref3d_f64* wk1, double dt,
                             const oeb_domain* dom, void* stream);

/* kernels/p_grad_c.h:4-6 -- p_grad_c(uout, vout, uin, vin, rdxc, rdyc, delpc, gz, pkc, wk, dt2) */
OEB_API oeb_status oeb_p_grad_c_f64(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                            const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref3d_f64* rdxc,
                            const oeb_memref3d_f64* rdyc, const oeb_memref3d_f64* delpc, const oeb_memref3d_f64* gz,
                            const oeb_memref3d_f64* pkc, double dt2, const oeb_domain* dom, void* stream);

/* kernels/fvtp2d.h:4-7 -- fvtp2d(q_i, q_j, fx1, fx2, fy1, fy2, q, crx, cry, ra_x, ra_y, xfx, yfx, area,
 *                                fxx, fyy, al, almq, br, b0, smt5); p1, p2 are the driver macros
 * (src/fvtp2d.cpp:11-12).  q_i, q_j, fx2 and fy2 are written over the same extended ranges as the
 * reference (fvtp2d.h:26-27, 46-47, 102-103, 122-123), so they need a 3-cell halo. */
OEB_API oeb_status oeb_fvtp2d_f64(const oeb_memref3d_f64* q_i, const oeb_memref3d_f64* q_j, const oeb_memref3d_f64* fx1,
                          const oeb_memref3d_f64* fx2, const oeb_memref3d_f64* fy1, const oeb_memref3d_f64* fy2,
                          const oeb_memref3d_f64* q, const oeb_memref3d_f64* crx, const oeb_memref3d_f64* cry,
                          const oeb_memref3d_f64* ra_x, const oeb_memref3d_f64* ra_y, const oeb_memref3d_f64* xfx,
                          const oeb_memref3d_f64* yfx, const oeb_memref3d_f64* area, double ppm_p1, double ppm_p2,
                          const oeb_domain* dom, void* stream);

/* ------------------------------------------------------------------------- */
/* FP64 forward stencils, HOST pointers, synchronous (see oeb_set_host_async). */
/* Same arguments as the device entry points; each call runs the kernels on    */
/* the host fields in place where the device can address them, else stages   */
/* its fields through device memory (inputs: the whole descriptor span;       */
/* outputs: exactly the written box), and returns once the outputs are in     */
/* host memory.  Any host memory works; pinned memory makes the copies DMA.   */
/* ------------------------------------------------------------------------- */

OEB_API oeb_status oeb_laplace_f64_host(const oeb_memref3d_f64* in, const oeb_memref3d_f64* out,
                                        const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hdiffsa_f64_host(const oeb_memref3d_f64* out, const oeb_memref3d_f64* in,
                                        const oeb_memref3d_f64* mask, const oeb_memref1d_f64* crlato,
                                        const oeb_memref1d_f64* crlatu, const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hdiffsmag_f64_host(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                                          const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                                          const oeb_memref3d_f64* mask, const oeb_memref1d_f64* crlavo,
                                          const oeb_memref1d_f64* crlavu, const oeb_memref1d_f64* crlato,
                                          const oeb_memref1d_f64* crlatu, const oeb_memref1d_f64* acrlat0,
                                          double eddlat, double eddlon, double tau_smag, double weight_smag,
                                          const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hadvuv_f64_host(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                                       const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                                       const oeb_memref1d_f64* acrlat0, const oeb_memref1d_f64* acrlat1,
                                       const oeb_memref1d_f64* tgrlatda0, const oeb_memref1d_f64* tgrlatda1,
                                       double eddlat, double eddlon, const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hadvuv5th_f64_host(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                                          const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                                          const oeb_memref1d_f64* acrlat0, const oeb_memref1d_f64* acrlat1,
                                          const oeb_memref1d_f64* tgrlatda0, const oeb_memref1d_f64* tgrlatda1,
                                          double eddlat, double eddlon, const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_fastwavesuv_f64_host(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                                            const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                                            const oeb_memref3d_f64* utens, const oeb_memref3d_f64* vtens,
                                            const oeb_memref3d_f64* wgtfac, const oeb_memref3d_f64* ppuv,
                                            const oeb_memref3d_f64* hhl, const oeb_memref3d_f64* rho,
                                            const oeb_memref1d_f64* fx, double edadlat, double dt,
                                            const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_uvbke_f64_host(const oeb_memref3d_f64* ub, const oeb_memref3d_f64* vb,
                                      const oeb_memref3d_f64* uc, const oeb_memref3d_f64* vc,
                                      const oeb_memref3d_f64* cosa, const oeb_memref3d_f64* rsina, double dt5,
                                      const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_nh_p_grad_f64_host(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                                          const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                                          const oeb_memref3d_f64* rdx, const oeb_memref3d_f64* rdy,
                                          const oeb_memref3d_f64* gz, const oeb_memref3d_f64* pp,
                                          const oeb_memref3d_f64* pk3, const oeb_memref3d_f64* wk1, double dt,
                                          const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_p_grad_c_f64_host(const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                                         const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin,
                                         const oeb_memref3d_f64* rdxc, const oeb_memref3d_f64* rdyc,
                                         const oeb_memref3d_f64* delpc, const oeb_memref3d_f64* gz,
                                         const oeb_memref3d_f64* pkc, double dt2, const oeb_domain* dom,
                                         void* stream);
OEB_API oeb_status oeb_fvtp2d_f64_host(const oeb_memref3d_f64* q_i, const oeb_memref3d_f64* q_j,
                                       const oeb_memref3d_f64* fx1, const oeb_memref3d_f64* fx2,
                                       const oeb_memref3d_f64* fy1, const oeb_memref3d_f64* fy2,
                                       const oeb_memref3d_f64* q, const oeb_memref3d_f64* crx,
                                       const oeb_memref3d_f64* cry, const oeb_memref3d_f64* ra_x,
                                       const oeb_memref3d_f64* ra_y, const oeb_memref3d_f64* xfx,
                                       const oeb_memref3d_f64* yfx, const oeb_memref3d_f64* area, double ppm_p1,
                                       double ppm_p2, const oeb_domain* dom, void* stream);


/* ------------------------------------------------------------------------- */
/* FP32 forward stencils: fields stored and computed in FP32.  Same arguments */
/* as the FP64 entry points with float scalars (dt5 stays a double, as in     */
/* the reference, src/uvbke.cpp:11-12).  Branch tests on the sign of a        */
/* product (hdiffsa limiter, fvtp2d PPM flag) are decided on the exact        */
/* product, and the hdiffsmag and advection flux sums are compensated, so the */
/* results differ from the FP64 ones only by FP32 rounding of the data; they  */
/* are not the reference compiled with ElementType = float.                   */
/* ------------------------------------------------------------------------- */

/* FP32 of kernels/laplace.h:4 -- laplace(in, out) */
OEB_API oeb_status oeb_laplace_f32(const oeb_memref3d_f32* in, const oeb_memref3d_f32* out, const oeb_domain* dom,
                           void* stream);

/* FP32 of kernels/hdiffsa.h:4-5 -- hdiffsa(out, in, mask, crlato, crlatu, lap, flx, fly) */
OEB_API oeb_status oeb_hdiffsa_f32(const oeb_memref3d_f32* out, const oeb_memref3d_f32* in, const oeb_memref3d_f32* mask,
                           const oeb_memref1d_f32* crlato, const oeb_memref1d_f32* crlatu, const oeb_domain* dom,
                           void* stream);

/* FP32 of kernels/hdiffsmag.h:4-7 -- hdiffsmag(uout, vout, uin, vin, mask, crlavo, crlavu, crlato, crlatu,
 *                                      acrlat0, T_sqr_s, S_sqr_uv, eddlat, eddlon, tau_smag, weight_smag) */
OEB_API oeb_status oeb_hdiffsmag_f32(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                             const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                             const oeb_memref3d_f32* mask, const oeb_memref1d_f32* crlavo,
                             const oeb_memref1d_f32* crlavu, const oeb_memref1d_f32* crlato,
                             const oeb_memref1d_f32* crlatu, const oeb_memref1d_f32* acrlat0, float eddlat,
                             float eddlon, float tau_smag, float weight_smag, const oeb_domain* dom,
                             void* stream);

/* FP32 of kernels/hadvuv.h:29-32 -- hadvuv(uout, vout, uin, vin, acrlat0, acrlat1, tgrlatda0, tgrlatda1,
 *                                  uatupos, vatupos, uatvpos, vatvpos, uavg, vavg, ures, vres, eddlat, eddlon) */
OEB_API oeb_status oeb_hadvuv_f32(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout, const oeb_memref3d_f32* uin,
                          const oeb_memref3d_f32* vin, const oeb_memref1d_f32* acrlat0,
                          const oeb_memref1d_f32* acrlat1, const oeb_memref1d_f32* tgrlatda0,
                          const oeb_memref1d_f32* tgrlatda1, float eddlat, float eddlon, const oeb_domain* dom,
                          void* stream);

/* FP32 of kernels/hadvuv5th.h:41-44 -- hadvuv5th(same arguments as hadvuv) */
OEB_API oeb_status oeb_hadvuv5th_f32(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                             const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                             const oeb_memref1d_f32* acrlat0, const oeb_memref1d_f32* acrlat1,
                             const oeb_memref1d_f32* tgrlatda0, const oeb_memref1d_f32* tgrlatda1, float eddlat,
                             float eddlon, const oeb_domain* dom, void* stream);

/* FP32 of kernels/fastwavesuv.h:4-7 -- fastwavesuv(uout, vout, uin, vin, utens, vtens, wgtfac, ppuv, hhl, rho, fx,
 *                                          ppgk, ppgc, ppgu, ppgv, edadlat, dt) */
OEB_API oeb_status oeb_fastwavesuv_f32(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                               const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                               const oeb_memref3d_f32* utens, const oeb_memref3d_f32* vtens,
                               const oeb_memref3d_f32* wgtfac, const oeb_memref3d_f32* ppuv,
                               const oeb_memref3d_f32* hhl, const oeb_memref3d_f32* rho, const oeb_memref1d_f32* fx,
                               float edadlat, float dt, const oeb_domain* dom, void* stream);

/* FP32 of kernels/uvbke.h:4-5 -- uvbke(ub, vb, uc, vc, cosa, rsina); dt5 is the driver global (src/uvbke.cpp:11-12) */
OEB_API oeb_status oeb_uvbke_f32(const oeb_memref3d_f32* ub, const oeb_memref3d_f32* vb, const oeb_memref3d_f32* uc,
                         const oeb_memref3d_f32* vc, const oeb_memref3d_f32* cosa, const oeb_memref3d_f32* rsina,
                         double dt5, const oeb_domain* dom, void* stream);

/* FP32 of kernels/nh_p_grad.h:4-6 -- nh_p_grad(uout, vout, uin, vin, rdx, rdy, gz, pp, pk3, wk1, wk, du, dv, dt) */
OEB_API oeb_status oeb_nh_p_grad_f32(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                             const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref3d_f32* rdx,
                             const oeb_memref3d_f32* rdy, const oeb_memref3d_f32* gz, const oeb_memref3d_f32* pp,
                             const oeb_memref3d_f32* pk3, const oeb_memref3d_f32* wk1, float dt,
                             const oeb_domain* dom, void* stream);

/* FP32 of kernels/p_grad_c.h:4-6 -- p_grad_c(uout, vout, uin, vin, rdxc, rdyc, delpc, gz, pkc, wk, dt2) */
OEB_API oeb_status oeb_p_grad_c_f32(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                            const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref3d_f32* rdxc,
                            const oeb_memref3d_f32* rdyc, const oeb_memref3d_f32* delpc, const oeb_memref3d_f32* gz,
                            const oeb_memref3d_f32* pkc, float dt2, const oeb_domain* dom, void* stream);

/* FP32 pressure gradients on profile-relative fields (no reference counterpart; the same
 * stencils as oeb_p_grad_c_f32 / oeb_nh_p_grad_f32).  gz, pkc (p_grad_c) and gz, pp, pk3
 * (nh_p_grad) hold FP32 perturbations from an FP64 per-level base profile: the field's value at
 * interior level k is base[k] + field[k].  Each *_base is a DEVICE array of nz + 1 doubles
 * (interior levels 0 .. nz, the stencils read level k + 1).  Differences between levels then
 * take the base difference in FP64 (rounded once to FP32) and differences within a level the
 * perturbations alone, so the outputs keep the accuracy the FP32 storage of full-value fields
 * loses (their profiles nearly cancel in the stencils' differences).  Fields and checks as the
 * standard entries; OEB_ERR_NULL for a NULL base. */
OEB_API oeb_status oeb_p_grad_c_f32_profiled(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                             const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                                             const oeb_memref3d_f32* rdxc, const oeb_memref3d_f32* rdyc,
                                             const oeb_memref3d_f32* delpc, const oeb_memref3d_f32* gz,
                                             const oeb_memref3d_f32* pkc, const double* gz_base,
                                             const double* pkc_base, float dt2, const oeb_domain* dom,
                                             void* stream);
OEB_API oeb_status oeb_nh_p_grad_f32_profiled(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                              const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                                              const oeb_memref3d_f32* rdx, const oeb_memref3d_f32* rdy,
                                              const oeb_memref3d_f32* gz, const oeb_memref3d_f32* pp,
                                              const oeb_memref3d_f32* pk3, const oeb_memref3d_f32* wk1,
                                              const double* gz_base, const double* pp_base,
                                              const double* pk3_base, float dt, const oeb_domain* dom,
                                              void* stream);

/* FP32 of kernels/fvtp2d.h:4-7 -- fvtp2d(q_i, q_j, fx1, fx2, fy1, fy2, q, crx, cry, ra_x, ra_y, xfx, yfx, area,
 *                                fxx, fyy, al, almq, br, b0, smt5); p1, p2 are the driver macros
 * (src/fvtp2d.cpp:11-12).  q_i, q_j, fx2 and fy2 are written over the same extended ranges as the
 * reference (fvtp2d.h:26-27, 46-47, 102-103, 122-123), so they need a 3-cell halo. */
OEB_API oeb_status oeb_fvtp2d_f32(const oeb_memref3d_f32* q_i, const oeb_memref3d_f32* q_j, const oeb_memref3d_f32* fx1,
                          const oeb_memref3d_f32* fx2, const oeb_memref3d_f32* fy1, const oeb_memref3d_f32* fy2,
                          const oeb_memref3d_f32* q, const oeb_memref3d_f32* crx, const oeb_memref3d_f32* cry,
                          const oeb_memref3d_f32* ra_x, const oeb_memref3d_f32* ra_y, const oeb_memref3d_f32* xfx,
                          const oeb_memref3d_f32* yfx, const oeb_memref3d_f32* area, float ppm_p1, float ppm_p2,
                          const oeb_domain* dom, void* stream);


OEB_API oeb_status oeb_laplace_f32_host(const oeb_memref3d_f32* in, const oeb_memref3d_f32* out,
                                        const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hdiffsa_f32_host(const oeb_memref3d_f32* out, const oeb_memref3d_f32* in,
                                        const oeb_memref3d_f32* mask, const oeb_memref1d_f32* crlato,
                                        const oeb_memref1d_f32* crlatu, const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hdiffsmag_f32_host(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                          const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                                          const oeb_memref3d_f32* mask, const oeb_memref1d_f32* crlavo,
                                          const oeb_memref1d_f32* crlavu, const oeb_memref1d_f32* crlato,
                                          const oeb_memref1d_f32* crlatu, const oeb_memref1d_f32* acrlat0,
                                          float eddlat, float eddlon, float tau_smag, float weight_smag,
                                          const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hadvuv_f32_host(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                       const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                                       const oeb_memref1d_f32* acrlat0, const oeb_memref1d_f32* acrlat1,
                                       const oeb_memref1d_f32* tgrlatda0, const oeb_memref1d_f32* tgrlatda1,
                                       float eddlat, float eddlon, const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hadvuv5th_f32_host(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                          const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                                          const oeb_memref1d_f32* acrlat0, const oeb_memref1d_f32* acrlat1,
                                          const oeb_memref1d_f32* tgrlatda0, const oeb_memref1d_f32* tgrlatda1,
                                          float eddlat, float eddlon, const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_fastwavesuv_f32_host(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                            const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                                            const oeb_memref3d_f32* utens, const oeb_memref3d_f32* vtens,
                                            const oeb_memref3d_f32* wgtfac, const oeb_memref3d_f32* ppuv,
                                            const oeb_memref3d_f32* hhl, const oeb_memref3d_f32* rho,
                                            const oeb_memref1d_f32* fx, float edadlat, float dt,
                                            const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_uvbke_f32_host(const oeb_memref3d_f32* ub, const oeb_memref3d_f32* vb,
                                      const oeb_memref3d_f32* uc, const oeb_memref3d_f32* vc,
                                      const oeb_memref3d_f32* cosa, const oeb_memref3d_f32* rsina, double dt5,
                                      const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_nh_p_grad_f32_host(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                          const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                                          const oeb_memref3d_f32* rdx, const oeb_memref3d_f32* rdy,
                                          const oeb_memref3d_f32* gz, const oeb_memref3d_f32* pp,
                                          const oeb_memref3d_f32* pk3, const oeb_memref3d_f32* wk1, float dt,
                                          const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_p_grad_c_f32_host(const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                         const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin,
                                         const oeb_memref3d_f32* rdxc, const oeb_memref3d_f32* rdyc,
                                         const oeb_memref3d_f32* delpc, const oeb_memref3d_f32* gz,
                                         const oeb_memref3d_f32* pkc, float dt2, const oeb_domain* dom,
                                         void* stream);
OEB_API oeb_status oeb_fvtp2d_f32_host(const oeb_memref3d_f32* q_i, const oeb_memref3d_f32* q_j,
                                       const oeb_memref3d_f32* fx1, const oeb_memref3d_f32* fx2,
                                       const oeb_memref3d_f32* fy1, const oeb_memref3d_f32* fy2,
                                       const oeb_memref3d_f32* q, const oeb_memref3d_f32* crx,
                                       const oeb_memref3d_f32* cry, const oeb_memref3d_f32* ra_x,
                                       const oeb_memref3d_f32* ra_y, const oeb_memref3d_f32* xfx,
                                       const oeb_memref3d_f32* yfx, const oeb_memref3d_f32* area, float ppm_p1,
                                       float ppm_p2, const oeb_domain* dom, void* stream);



/* ------------------------------------------------------------------------- */
/* Tangent-linear stencils: dy = J(x) dx, the Jacobian of the forward stencil */
/* at the state x (every upwind/limiter/PPM/clamp branch frozen at x) applied */
/* to a perturbation dx of the active inputs.  Device pointers, asynchronous; */
/* each dx field must have the layout of its state field.  dy is written over */
/* the forward output's written box.  Device scratch from the library pool.   */
/*   hdiffsmag, hadvuv, hadvuv5th : active (uin, vin)                          */
/*   fastwavesuv                  : active (uin, vin, utens, vtens, ppuv)      */
/*   fvtp2d                       : active q; dy = all six outputs            */
/*   laplace, hdiffsa             : active in                                 */
/*   uvbke                        : active (uc, vc)                           */
/*   nh_p_grad                    : active (uin, vin, gz, pp, pk3, wk1)       */
/*   p_grad_c                     : active (uin, vin, delpc, gz, pkc)         */
/* Argument order: dy for every output, the forward inputs in the reference    */
/* signature's order, dx for every active input, the scalars.                 */
/* ------------------------------------------------------------------------- */

OEB_API oeb_status oeb_hdiffsmag_tl_f64(const oeb_memref3d_f64* duout, const oeb_memref3d_f64* dvout, const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref3d_f64* mask,
                                       const oeb_memref1d_f64* crlavo, const oeb_memref1d_f64* crlavu, const oeb_memref1d_f64* crlato, const oeb_memref1d_f64* crlatu, const oeb_memref1d_f64* acrlat0,
                                       const oeb_memref3d_f64* duin, const oeb_memref3d_f64* dvin, double eddlat, double eddlon, double tau_smag, double weight_smag,
                                       const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hadvuv_tl_f64(const oeb_memref3d_f64* duout, const oeb_memref3d_f64* dvout, const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref1d_f64* acrlat0, const oeb_memref1d_f64* acrlat1,
                                    const oeb_memref1d_f64* tgrlatda0, const oeb_memref1d_f64* tgrlatda1, const oeb_memref3d_f64* duin, const oeb_memref3d_f64* dvin, double eddlat, double eddlon,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hadvuv5th_tl_f64(const oeb_memref3d_f64* duout, const oeb_memref3d_f64* dvout, const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref1d_f64* acrlat0, const oeb_memref1d_f64* acrlat1,
                                       const oeb_memref1d_f64* tgrlatda0, const oeb_memref1d_f64* tgrlatda1, const oeb_memref3d_f64* duin, const oeb_memref3d_f64* dvin, double eddlat, double eddlon,
                                       const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_fastwavesuv_tl_f64(const oeb_memref3d_f64* duout, const oeb_memref3d_f64* dvout, const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref3d_f64* utens, const oeb_memref3d_f64* vtens,
                                         const oeb_memref3d_f64* wgtfac, const oeb_memref3d_f64* ppuv, const oeb_memref3d_f64* hhl, const oeb_memref3d_f64* rho, const oeb_memref1d_f64* fx, const oeb_memref3d_f64* duin, const oeb_memref3d_f64* dvin,
                                         const oeb_memref3d_f64* dutens, const oeb_memref3d_f64* dvtens, const oeb_memref3d_f64* dppuv, double edadlat, double dt,
                                         const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_fvtp2d_tl_f64(const oeb_memref3d_f64* dq_i, const oeb_memref3d_f64* dq_j, const oeb_memref3d_f64* dfx1, const oeb_memref3d_f64* dfx2, const oeb_memref3d_f64* dfy1, const oeb_memref3d_f64* dfy2, const oeb_memref3d_f64* q,
                                    const oeb_memref3d_f64* crx, const oeb_memref3d_f64* cry, const oeb_memref3d_f64* ra_x, const oeb_memref3d_f64* ra_y, const oeb_memref3d_f64* xfx, const oeb_memref3d_f64* yfx, const oeb_memref3d_f64* area,
                                    const oeb_memref3d_f64* dq, double ppm_p1, double ppm_p2, const oeb_domain* dom, void* stream);

/* kernels/laplace.h:34-43, hdiffsa.h:95-123, uvbke.h:61-75, nh_p_grad.h:116-146, p_grad_c.h:80-101 */
OEB_API oeb_status oeb_laplace_tl_f64(const oeb_memref3d_f64* dout, const oeb_memref3d_f64* in, const oeb_memref3d_f64* din,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hdiffsa_tl_f64(const oeb_memref3d_f64* dout, const oeb_memref3d_f64* in, const oeb_memref3d_f64* mask, const oeb_memref1d_f64* crlato, const oeb_memref1d_f64* crlatu, const oeb_memref3d_f64* din,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_uvbke_tl_f64(const oeb_memref3d_f64* dub, const oeb_memref3d_f64* dvb, const oeb_memref3d_f64* uc, const oeb_memref3d_f64* vc, const oeb_memref3d_f64* cosa, const oeb_memref3d_f64* rsina, const oeb_memref3d_f64* duc, const oeb_memref3d_f64* dvc, double dt5,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_nh_p_grad_tl_f64(const oeb_memref3d_f64* duout, const oeb_memref3d_f64* dvout, const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref3d_f64* rdx, const oeb_memref3d_f64* rdy, const oeb_memref3d_f64* gz, const oeb_memref3d_f64* pp, const oeb_memref3d_f64* pk3, const oeb_memref3d_f64* wk1, const oeb_memref3d_f64* duin, const oeb_memref3d_f64* dvin, const oeb_memref3d_f64* dgz, const oeb_memref3d_f64* dpp, const oeb_memref3d_f64* dpk3, const oeb_memref3d_f64* dwk1, double dt,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_p_grad_c_tl_f64(const oeb_memref3d_f64* duout, const oeb_memref3d_f64* dvout, const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref3d_f64* rdxc, const oeb_memref3d_f64* rdyc, const oeb_memref3d_f64* delpc, const oeb_memref3d_f64* gz, const oeb_memref3d_f64* pkc, const oeb_memref3d_f64* duin, const oeb_memref3d_f64* dvin, const oeb_memref3d_f64* ddelpc, const oeb_memref3d_f64* dgz, const oeb_memref3d_f64* dpkc, double dt2,
                                    const oeb_domain* dom, void* stream);

OEB_API oeb_status oeb_hdiffsmag_tl_f32(const oeb_memref3d_f32* duout, const oeb_memref3d_f32* dvout, const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref3d_f32* mask,
                                       const oeb_memref1d_f32* crlavo, const oeb_memref1d_f32* crlavu, const oeb_memref1d_f32* crlato, const oeb_memref1d_f32* crlatu, const oeb_memref1d_f32* acrlat0,
                                       const oeb_memref3d_f32* duin, const oeb_memref3d_f32* dvin, float eddlat, float eddlon, float tau_smag, float weight_smag,
                                       const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hadvuv_tl_f32(const oeb_memref3d_f32* duout, const oeb_memref3d_f32* dvout, const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref1d_f32* acrlat0, const oeb_memref1d_f32* acrlat1,
                                    const oeb_memref1d_f32* tgrlatda0, const oeb_memref1d_f32* tgrlatda1, const oeb_memref3d_f32* duin, const oeb_memref3d_f32* dvin, float eddlat, float eddlon,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hadvuv5th_tl_f32(const oeb_memref3d_f32* duout, const oeb_memref3d_f32* dvout, const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref1d_f32* acrlat0, const oeb_memref1d_f32* acrlat1,
                                       const oeb_memref1d_f32* tgrlatda0, const oeb_memref1d_f32* tgrlatda1, const oeb_memref3d_f32* duin, const oeb_memref3d_f32* dvin, float eddlat, float eddlon,
                                       const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_fastwavesuv_tl_f32(const oeb_memref3d_f32* duout, const oeb_memref3d_f32* dvout, const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref3d_f32* utens, const oeb_memref3d_f32* vtens,
                                         const oeb_memref3d_f32* wgtfac, const oeb_memref3d_f32* ppuv, const oeb_memref3d_f32* hhl, const oeb_memref3d_f32* rho, const oeb_memref1d_f32* fx, const oeb_memref3d_f32* duin, const oeb_memref3d_f32* dvin,
                                         const oeb_memref3d_f32* dutens, const oeb_memref3d_f32* dvtens, const oeb_memref3d_f32* dppuv, float edadlat, float dt,
                                         const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_fvtp2d_tl_f32(const oeb_memref3d_f32* dq_i, const oeb_memref3d_f32* dq_j, const oeb_memref3d_f32* dfx1, const oeb_memref3d_f32* dfx2, const oeb_memref3d_f32* dfy1, const oeb_memref3d_f32* dfy2, const oeb_memref3d_f32* q,
                                    const oeb_memref3d_f32* crx, const oeb_memref3d_f32* cry, const oeb_memref3d_f32* ra_x, const oeb_memref3d_f32* ra_y, const oeb_memref3d_f32* xfx, const oeb_memref3d_f32* yfx, const oeb_memref3d_f32* area,
                                    const oeb_memref3d_f32* dq, float ppm_p1, float ppm_p2, const oeb_domain* dom, void* stream);

/* kernels/laplace.h:34-43, hdiffsa.h:95-123, uvbke.h:61-75, nh_p_grad.h:116-146, p_grad_c.h:80-101 */
OEB_API oeb_status oeb_laplace_tl_f32(const oeb_memref3d_f32* dout, const oeb_memref3d_f32* in, const oeb_memref3d_f32* din,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hdiffsa_tl_f32(const oeb_memref3d_f32* dout, const oeb_memref3d_f32* in, const oeb_memref3d_f32* mask, const oeb_memref1d_f32* crlato, const oeb_memref1d_f32* crlatu, const oeb_memref3d_f32* din,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_uvbke_tl_f32(const oeb_memref3d_f32* dub, const oeb_memref3d_f32* dvb, const oeb_memref3d_f32* uc, const oeb_memref3d_f32* vc, const oeb_memref3d_f32* cosa, const oeb_memref3d_f32* rsina, const oeb_memref3d_f32* duc, const oeb_memref3d_f32* dvc, double dt5,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_nh_p_grad_tl_f32(const oeb_memref3d_f32* duout, const oeb_memref3d_f32* dvout, const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref3d_f32* rdx, const oeb_memref3d_f32* rdy, const oeb_memref3d_f32* gz, const oeb_memref3d_f32* pp, const oeb_memref3d_f32* pk3, const oeb_memref3d_f32* wk1, const oeb_memref3d_f32* duin, const oeb_memref3d_f32* dvin, const oeb_memref3d_f32* dgz, const oeb_memref3d_f32* dpp, const oeb_memref3d_f32* dpk3, const oeb_memref3d_f32* dwk1, float dt,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_p_grad_c_tl_f32(const oeb_memref3d_f32* duout, const oeb_memref3d_f32* dvout, const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref3d_f32* rdxc, const oeb_memref3d_f32* rdyc, const oeb_memref3d_f32* delpc, const oeb_memref3d_f32* gz, const oeb_memref3d_f32* pkc, const oeb_memref3d_f32* duin, const oeb_memref3d_f32* dvin, const oeb_memref3d_f32* ddelpc, const oeb_memref3d_f32* dgz, const oeb_memref3d_f32* dpkc, float dt2,
                                    const oeb_domain* dom, void* stream);


/* ------------------------------------------------------------------------- */
/* Adjoint (transpose) stencils: xb = J(x)^T yb, the transpose of the         */
/* tangent-linear map above at the state x, branches frozen at x.  Written    */
/* as gathers (no atomics) over per-point terms recomputed from the state,    */
/* in device scratch from the library pool.  Each xb is written over the      */
/* reach box of its input (the cells its forward output depends on) and is    */
/* overwritten, not accumulated.  Device pointers, asynchronous.              */
/*   hdiffsmag: xb = (uinb, vinb) on halo 1;  hadvuv / hadvuv5th: halo 2 / 3  */
/*   fastwavesuv: uinb, vinb, utensb, vtensb on the interior, ppuvb on        */
/*     i,j in [0,N], k in [-1,N_z];  fvtp2d: qb on halo 3 from (fx1b, fy1b)   */
/*   laplace: inb on halo 1;  hdiffsa: inb on halo 2 (limiters frozen)       */
/*   uvbke: ucb on i in [0,N), j in [-1,N); vcb on i in [-1,N), j in [0,N)   */
/*   nh_p_grad: uinb, vinb on the interior; gzb, ppb, pk3b on i,j in [0,N],  */
/*     k in [0,N_z]; wk1b on i,j in [0,N]                                     */
/*   p_grad_c: uinb, vinb on the interior; delpcb on i,j in [-1,N); gzb,     */
/*     pkcb on i,j in [-1,N), k in [0,N_z]                                    */
/* Argument order: xb for every active input, the forward inputs in the       */
/* reference signature's order, yb for every semantic output, the scalars.    */
/* ------------------------------------------------------------------------- */

/* kernels/laplace.h:34-43, hdiffsa.h:95-123, uvbke.h:61-75, nh_p_grad.h:116-146, p_grad_c.h:80-101 */
OEB_API oeb_status oeb_laplace_adj_f64(const oeb_memref3d_f64* inb, const oeb_memref3d_f64* in, const oeb_memref3d_f64* outb,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hdiffsa_adj_f64(const oeb_memref3d_f64* inb, const oeb_memref3d_f64* in, const oeb_memref3d_f64* mask, const oeb_memref1d_f64* crlato, const oeb_memref1d_f64* crlatu, const oeb_memref3d_f64* outb,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_uvbke_adj_f64(const oeb_memref3d_f64* ucb, const oeb_memref3d_f64* vcb, const oeb_memref3d_f64* uc, const oeb_memref3d_f64* vc, const oeb_memref3d_f64* cosa, const oeb_memref3d_f64* rsina, const oeb_memref3d_f64* ubb, const oeb_memref3d_f64* vbb, double dt5,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_nh_p_grad_adj_f64(const oeb_memref3d_f64* uinb, const oeb_memref3d_f64* vinb, const oeb_memref3d_f64* gzb, const oeb_memref3d_f64* ppb, const oeb_memref3d_f64* pk3b, const oeb_memref3d_f64* wk1b, const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref3d_f64* rdx, const oeb_memref3d_f64* rdy, const oeb_memref3d_f64* gz, const oeb_memref3d_f64* pp, const oeb_memref3d_f64* pk3, const oeb_memref3d_f64* wk1, const oeb_memref3d_f64* uoutb, const oeb_memref3d_f64* voutb, double dt,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_p_grad_c_adj_f64(const oeb_memref3d_f64* uinb, const oeb_memref3d_f64* vinb, const oeb_memref3d_f64* delpcb, const oeb_memref3d_f64* gzb, const oeb_memref3d_f64* pkcb, const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref3d_f64* rdxc, const oeb_memref3d_f64* rdyc, const oeb_memref3d_f64* delpc, const oeb_memref3d_f64* gz, const oeb_memref3d_f64* pkc, const oeb_memref3d_f64* uoutb, const oeb_memref3d_f64* voutb, double dt2,
                                    const oeb_domain* dom, void* stream);

OEB_API oeb_status oeb_hdiffsmag_adj_f64(const oeb_memref3d_f64* uinb, const oeb_memref3d_f64* vinb, const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref3d_f64* mask, const oeb_memref1d_f64* crlavo,
                                        const oeb_memref1d_f64* crlavu, const oeb_memref1d_f64* crlato, const oeb_memref1d_f64* crlatu, const oeb_memref1d_f64* acrlat0, const oeb_memref3d_f64* uoutb,
                                        const oeb_memref3d_f64* voutb, double eddlat, double eddlon, double tau_smag, double weight_smag,
                                        const oeb_domain* dom, void* stream);
/* No counterpart in the reference.  oeb_hdiffsmag_adj_f64 without any allocation: the same   */
/* arguments, checks and results, with its scratch in one fixed array inside the library,     */
/* for callers that cannot allocate device memory while they run (a host whose allocator has  */
/* claimed the GPU's memory up front, or a step loop that must not allocate).  Limit: uin's  */
/* allocation span (halo and padding included) at most 2^21 cells, else OEB_ERR_TOO_LARGE    */
/* before anything runs; the array (96 MiB) is held on every GPU that loads the library until */
/* the process exits.  All calls share it and it keeps the last call's contents (nothing in   */
/* it needs to start at zero); calls that overlap on the GPU race.  The first call on a       */
/* device looks up the array's device address with that device current: make that first call */
/* before any stream capture.  The address is kept for the life of the process, so do not     */
/* call this entry point on a device after cudaDeviceReset of that device.                    */
OEB_API oeb_status oeb_hdiffsmag_adj_noalloc_f64(const oeb_memref3d_f64* uinb, const oeb_memref3d_f64* vinb, const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref3d_f64* mask,
                                                const oeb_memref1d_f64* crlavo, const oeb_memref1d_f64* crlavu, const oeb_memref1d_f64* crlato, const oeb_memref1d_f64* crlatu,
                                                const oeb_memref1d_f64* acrlat0, const oeb_memref3d_f64* uoutb, const oeb_memref3d_f64* voutb, double eddlat, double eddlon,
                                                double tau_smag, double weight_smag, const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hadvuv_adj_f64(const oeb_memref3d_f64* uinb, const oeb_memref3d_f64* vinb, const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref1d_f64* acrlat0, const oeb_memref1d_f64* acrlat1,
                                     const oeb_memref1d_f64* tgrlatda0, const oeb_memref1d_f64* tgrlatda1, const oeb_memref3d_f64* uoutb, const oeb_memref3d_f64* voutb, double eddlat,
                                     double eddlon, const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hadvuv5th_adj_f64(const oeb_memref3d_f64* uinb, const oeb_memref3d_f64* vinb, const oeb_memref3d_f64* uin, const oeb_memref3d_f64* vin, const oeb_memref1d_f64* acrlat0, const oeb_memref1d_f64* acrlat1,
                                        const oeb_memref1d_f64* tgrlatda0, const oeb_memref1d_f64* tgrlatda1, const oeb_memref3d_f64* uoutb, const oeb_memref3d_f64* voutb, double eddlat,
                                        double eddlon, const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_fastwavesuv_adj_f64(const oeb_memref3d_f64* uinb, const oeb_memref3d_f64* vinb, const oeb_memref3d_f64* utensb, const oeb_memref3d_f64* vtensb, const oeb_memref3d_f64* ppuvb, const oeb_memref3d_f64* uin,
                                          const oeb_memref3d_f64* vin, const oeb_memref3d_f64* utens, const oeb_memref3d_f64* vtens, const oeb_memref3d_f64* wgtfac, const oeb_memref3d_f64* ppuv, const oeb_memref3d_f64* hhl,
                                          const oeb_memref3d_f64* rho, const oeb_memref1d_f64* fx, const oeb_memref3d_f64* uoutb, const oeb_memref3d_f64* voutb, double edadlat, double dt,
                                          const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_fvtp2d_adj_f64(const oeb_memref3d_f64* qb, const oeb_memref3d_f64* q, const oeb_memref3d_f64* crx, const oeb_memref3d_f64* cry, const oeb_memref3d_f64* ra_x, const oeb_memref3d_f64* ra_y, const oeb_memref3d_f64* xfx,
                                     const oeb_memref3d_f64* yfx, const oeb_memref3d_f64* area, const oeb_memref3d_f64* fx1b, const oeb_memref3d_f64* fy1b, double ppm_p1, double ppm_p2,
                                     const oeb_domain* dom, void* stream);

/* kernels/laplace.h:34-43, hdiffsa.h:95-123, uvbke.h:61-75, nh_p_grad.h:116-146, p_grad_c.h:80-101 */
OEB_API oeb_status oeb_laplace_adj_f32(const oeb_memref3d_f32* inb, const oeb_memref3d_f32* in, const oeb_memref3d_f32* outb,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hdiffsa_adj_f32(const oeb_memref3d_f32* inb, const oeb_memref3d_f32* in, const oeb_memref3d_f32* mask, const oeb_memref1d_f32* crlato, const oeb_memref1d_f32* crlatu, const oeb_memref3d_f32* outb,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_uvbke_adj_f32(const oeb_memref3d_f32* ucb, const oeb_memref3d_f32* vcb, const oeb_memref3d_f32* uc, const oeb_memref3d_f32* vc, const oeb_memref3d_f32* cosa, const oeb_memref3d_f32* rsina, const oeb_memref3d_f32* ubb, const oeb_memref3d_f32* vbb, double dt5,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_nh_p_grad_adj_f32(const oeb_memref3d_f32* uinb, const oeb_memref3d_f32* vinb, const oeb_memref3d_f32* gzb, const oeb_memref3d_f32* ppb, const oeb_memref3d_f32* pk3b, const oeb_memref3d_f32* wk1b, const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref3d_f32* rdx, const oeb_memref3d_f32* rdy, const oeb_memref3d_f32* gz, const oeb_memref3d_f32* pp, const oeb_memref3d_f32* pk3, const oeb_memref3d_f32* wk1, const oeb_memref3d_f32* uoutb, const oeb_memref3d_f32* voutb, float dt,
                                    const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_p_grad_c_adj_f32(const oeb_memref3d_f32* uinb, const oeb_memref3d_f32* vinb, const oeb_memref3d_f32* delpcb, const oeb_memref3d_f32* gzb, const oeb_memref3d_f32* pkcb, const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref3d_f32* rdxc, const oeb_memref3d_f32* rdyc, const oeb_memref3d_f32* delpc, const oeb_memref3d_f32* gz, const oeb_memref3d_f32* pkc, const oeb_memref3d_f32* uoutb, const oeb_memref3d_f32* voutb, float dt2,
                                    const oeb_domain* dom, void* stream);

OEB_API oeb_status oeb_hdiffsmag_adj_f32(const oeb_memref3d_f32* uinb, const oeb_memref3d_f32* vinb, const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref3d_f32* mask, const oeb_memref1d_f32* crlavo,
                                        const oeb_memref1d_f32* crlavu, const oeb_memref1d_f32* crlato, const oeb_memref1d_f32* crlatu, const oeb_memref1d_f32* acrlat0, const oeb_memref3d_f32* uoutb,
                                        const oeb_memref3d_f32* voutb, float eddlat, float eddlon, float tau_smag, float weight_smag,
                                        const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hadvuv_adj_f32(const oeb_memref3d_f32* uinb, const oeb_memref3d_f32* vinb, const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref1d_f32* acrlat0, const oeb_memref1d_f32* acrlat1,
                                     const oeb_memref1d_f32* tgrlatda0, const oeb_memref1d_f32* tgrlatda1, const oeb_memref3d_f32* uoutb, const oeb_memref3d_f32* voutb, float eddlat,
                                     float eddlon, const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_hadvuv5th_adj_f32(const oeb_memref3d_f32* uinb, const oeb_memref3d_f32* vinb, const oeb_memref3d_f32* uin, const oeb_memref3d_f32* vin, const oeb_memref1d_f32* acrlat0, const oeb_memref1d_f32* acrlat1,
                                        const oeb_memref1d_f32* tgrlatda0, const oeb_memref1d_f32* tgrlatda1, const oeb_memref3d_f32* uoutb, const oeb_memref3d_f32* voutb, float eddlat,
                                        float eddlon, const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_fastwavesuv_adj_f32(const oeb_memref3d_f32* uinb, const oeb_memref3d_f32* vinb, const oeb_memref3d_f32* utensb, const oeb_memref3d_f32* vtensb, const oeb_memref3d_f32* ppuvb, const oeb_memref3d_f32* uin,
                                          const oeb_memref3d_f32* vin, const oeb_memref3d_f32* utens, const oeb_memref3d_f32* vtens, const oeb_memref3d_f32* wgtfac, const oeb_memref3d_f32* ppuv, const oeb_memref3d_f32* hhl,
                                          const oeb_memref3d_f32* rho, const oeb_memref1d_f32* fx, const oeb_memref3d_f32* uoutb, const oeb_memref3d_f32* voutb, float edadlat, float dt,
                                          const oeb_domain* dom, void* stream);
OEB_API oeb_status oeb_fvtp2d_adj_f32(const oeb_memref3d_f32* qb, const oeb_memref3d_f32* q, const oeb_memref3d_f32* crx, const oeb_memref3d_f32* cry, const oeb_memref3d_f32* ra_x, const oeb_memref3d_f32* ra_y, const oeb_memref3d_f32* xfx,
                                     const oeb_memref3d_f32* yfx, const oeb_memref3d_f32* area, const oeb_memref3d_f32* fx1b, const oeb_memref3d_f32* fy1b, float ppm_p1, float ppm_p2,
                                     const oeb_domain* dom, void* stream);

/* ------------------------------------------------------------------------- */
/* Chained dycore step (no counterpart in the reference: its drivers,        */
/* src/<k>.cpp, run each stencil alone).  One step maps (u, v) to            */
/* (uout, vout, fx1, fy1):                                                   */
/*   1. (u1, v1)     = fastwavesuv(u, v, utens, vtens, wgtfac, ppuv, hhl,      */
/*                                 rho, fx; edadlat, dt)                     */
/*   2. (tu, tv)     = hadvuv5th(u1, v1, acrlat0, acrlat1, tgrlatda0,          */
/*                               tgrlatda1; eddlat, eddlon)                  */
/*   3. (u2, v2)     = (u1 + dt_adv tu, v1 + dt_adv tv)                       */
/*   4. (uout, vout) = hdiffsmag(u2, v2, mask, crlavo, crlavu, crlato, crlatu,  */
/*                               smag_acrlat0; eddlat, eddlon, tau_smag,     */
/*                               weight_smag)                                */
/*   5. (fx1, fy1)   = fvtp2d(q = uout, crx, cry, ra_x, ra_y, xfx, yfx, area;    */
/*                            ppm_p1, ppm_p2): PPM fluxes of the new u       */
/* Stage s runs over the interior widened in i and j by what the later        */
/* stages read (7, 4, 4, 3 and 0 cells), so one step needs no halo exchange:  */
/* the inputs need an i/j halo of 8 (7 below, 8 above for wgtfac, ppuv, hhl,  */
/* rho; 7 for the 1-D fields) and a k halo of 1; uout and vout are written    */
/* over the interior widened by 3, fx1 and fy1 over the interior.             */
/*                                                                           */
/* The tangent-linear step maps (du, dv) to (duout, dvout, dfx1, dfy1); the   */
/* adjoint maps (uoutb, voutb, fx1b, fy1b), seeds on the interior, to         */
/* (ub, vb) written over the interior widened by 7.  Both take only the      */
/* step's inputs: the intermediate states (u1, v1, u2, v2, the new u) are    */
/* recomputed inside the call, never stored between calls.                   */
/*                                                                           */
/* A plan owns the step's workspace: fields laid out like `like` (same        */
/* sizes, strides and offset, which every field of the step must share),     */
/* allocated once by oeb_chain_plan_create_* for the modes asked for, on the */
/* current device.  The step calls allocate only the scratch of the adjoint   */
/* and tangent-linear stencils they run (stream-ordered pool).  One plan      */
/* serves one stream at a time.                                              */
/* ------------------------------------------------------------------------- */
typedef struct oeb_chain_plan oeb_chain_plan;

#define OEB_CHAIN_FORWARD 1
#define OEB_CHAIN_TL 2
#define OEB_CHAIN_ADJOINT 4

typedef struct oeb_chain_fields_f64 {
  const oeb_memref3d_f64 *u, *v;
  const oeb_memref3d_f64 *utens, *vtens, *wgtfac, *ppuv, *hhl, *rho; /* fastwavesuv */
  const oeb_memref1d_f64* fx;
  const oeb_memref1d_f64 *acrlat0, *acrlat1, *tgrlatda0, *tgrlatda1; /* hadvuv5th */
  const oeb_memref3d_f64* mask;                                       /* hdiffsmag */
  const oeb_memref1d_f64 *crlavo, *crlavu, *crlato, *crlatu, *smag_acrlat0;
  const oeb_memref3d_f64 *crx, *cry, *ra_x, *ra_y, *xfx, *yfx, *area; /* fvtp2d */
} oeb_chain_fields_f64;

typedef struct oeb_chain_fields_f32 {
  const oeb_memref3d_f32 *u, *v;
  const oeb_memref3d_f32 *utens, *vtens, *wgtfac, *ppuv, *hhl, *rho;
  const oeb_memref1d_f32* fx;
  const oeb_memref1d_f32 *acrlat0, *acrlat1, *tgrlatda0, *tgrlatda1;
  const oeb_memref3d_f32* mask;
  const oeb_memref1d_f32 *crlavo, *crlavu, *crlato, *crlatu, *smag_acrlat0;
  const oeb_memref3d_f32 *crx, *cry, *ra_x, *ra_y, *xfx, *yfx, *area;
} oeb_chain_fields_f32;

/* Scalars of the step, in double; the FP32 step rounds them to float. */
typedef struct oeb_chain_scalars {
  double edadlat, dt;            /* fastwavesuv */
  double eddlat, eddlon;         /* hadvuv5th and hdiffsmag */
  double dt_adv;                 /* stage 3 */
  double tau_smag, weight_smag;  /* hdiffsmag */
  double ppm_p1, ppm_p2;         /* fvtp2d */
} oeb_chain_scalars;

OEB_API oeb_status oeb_chain_plan_create_f64(const oeb_memref3d_f64* like, const oeb_domain* dom, int modes,
                                             oeb_chain_plan** out);
OEB_API oeb_status oeb_chain_plan_create_f32(const oeb_memref3d_f32* like, const oeb_domain* dom, int modes,
                                             oeb_chain_plan** out);
/* Device bytes held by the plan's workspace. */
OEB_API size_t oeb_chain_plan_bytes(const oeb_chain_plan* plan);
/* Frees the workspace (after synchronising the device). */
OEB_API oeb_status oeb_chain_plan_destroy(oeb_chain_plan* plan);

OEB_API oeb_status oeb_chain_forward_f64(oeb_chain_plan* plan, const oeb_chain_fields_f64* f, const oeb_chain_scalars* s,
                                         const oeb_memref3d_f64* uout, const oeb_memref3d_f64* vout,
                                         const oeb_memref3d_f64* fx1, const oeb_memref3d_f64* fy1, void* stream);
OEB_API oeb_status oeb_chain_tl_f64(oeb_chain_plan* plan, const oeb_chain_fields_f64* f, const oeb_chain_scalars* s,
                                    const oeb_memref3d_f64* du, const oeb_memref3d_f64* dv,
                                    const oeb_memref3d_f64* duout, const oeb_memref3d_f64* dvout,
                                    const oeb_memref3d_f64* dfx1, const oeb_memref3d_f64* dfy1, void* stream);
OEB_API oeb_status oeb_chain_adj_f64(oeb_chain_plan* plan, const oeb_chain_fields_f64* f, const oeb_chain_scalars* s,
                                     const oeb_memref3d_f64* uoutb, const oeb_memref3d_f64* voutb,
                                     const oeb_memref3d_f64* fx1b, const oeb_memref3d_f64* fy1b,
                                     const oeb_memref3d_f64* ub, const oeb_memref3d_f64* vb, void* stream);
OEB_API oeb_status oeb_chain_forward_f32(oeb_chain_plan* plan, const oeb_chain_fields_f32* f, const oeb_chain_scalars* s,
                                         const oeb_memref3d_f32* uout, const oeb_memref3d_f32* vout,
                                         const oeb_memref3d_f32* fx1, const oeb_memref3d_f32* fy1, void* stream);
OEB_API oeb_status oeb_chain_tl_f32(oeb_chain_plan* plan, const oeb_chain_fields_f32* f, const oeb_chain_scalars* s,
                                    const oeb_memref3d_f32* du, const oeb_memref3d_f32* dv,
                                    const oeb_memref3d_f32* duout, const oeb_memref3d_f32* dvout,
                                    const oeb_memref3d_f32* dfx1, const oeb_memref3d_f32* dfy1, void* stream);
OEB_API oeb_status oeb_chain_adj_f32(oeb_chain_plan* plan, const oeb_chain_fields_f32* f, const oeb_chain_scalars* s,
                                     const oeb_memref3d_f32* uoutb, const oeb_memref3d_f32* voutb,
                                     const oeb_memref3d_f32* fx1b, const oeb_memref3d_f32* fy1b,
                                     const oeb_memref3d_f32* ub, const oeb_memref3d_f32* vb, void* stream);

/* ------------------------------------------------------------------------- */
/* Batched ensembles (no counterpart in the reference).  A batch plan runs    */
/* the chained step -- forward, then adjoint -- for many ensemble members of  */
/* uneven sizes and mixed precision.  At creation it records the step of    */
/* every member once (the calls of oeb_chain_forward_* / oeb_chain_adj_*,   */
/* launching nothing) and uploads, for each recorded kernel launch, the      */
/* members' tiles and arguments; oeb_batch_run then replays each launch as   */
/* ONE persistent kernel over all members of a precision, its CTAs walking   */
/* the (member, tile) items.  FP64 members run on `stream`, FP32 members on  */
/* a second stream of the plan that forks from and joins `stream`.  The     */
/* members' descriptors are baked in: a run reads and writes the same        */
/* buffers.  Each member has its own chain plan; the scratch of the adjoint  */
/* stencils lives in one arena of the plan.  Results are bit-identical to    */
/* oeb_chain_forward_* / oeb_chain_adj_* on each member.                     */
/*                                                                           */
/* oeb_batch_autotune times, for every batched launch, the k-levels per tile */
/* (kb) and the CTA count (one persistent wave, or one CTA per tile) and     */
/* keeps the fastest; oeb_batch_run uses the choices from then on.           */
/* ------------------------------------------------------------------------- */
typedef struct oeb_batch_plan oeb_batch_plan;

typedef struct oeb_batch_member {
  int elem_size;             /* 8: FP64 fields, 4: FP32 fields */
  oeb_domain dom;
  const void* fields;        /* const oeb_chain_fields_f64* or oeb_chain_fields_f32* */
  oeb_chain_scalars scalars;
  /* oeb_memref3d_f64 or _f32 descriptors */
  const void *uout, *vout, *fx1, *fy1;      /* forward outputs */
  const void *uoutb, *voutb, *fx1b, *fy1b;  /* adjoint seeds (OEB_CHAIN_ADJOINT) */
  const void *ub, *vb;                      /* adjoint results (OEB_CHAIN_ADJOINT) */
} oeb_batch_member;

/* modes: OEB_CHAIN_FORWARD and/or OEB_CHAIN_ADJOINT. */
OEB_API oeb_status oeb_batch_plan_create(const oeb_batch_member* members, int count, int modes, oeb_batch_plan** out);
OEB_API oeb_status oeb_batch_run(oeb_batch_plan* plan, void* stream);
OEB_API oeb_status oeb_batch_autotune(oeb_batch_plan* plan, void* stream);
/* Tuning records (no counterpart in the reference: its drivers take no tuning).  A record
 * keeps the autotuner's choices, so that a later process can apply them to a plan over the
 * same ensemble without timing anything again.  It holds three ints per batched launch, in
 * run order: kb (0 = each kernel's default, or 1, 2, 4, 8), the tile shape (0, 1, 2 as for
 * oeb_set_tile_shape; kernels without shapes ignore it) and the launch form (0: one
 * persistent wave, sized on the device it is applied on; 1: one CTA per tile; 2: one
 * ordinary launch per member).
 * oeb_batch_autotune times, for every launch, each kb with each tile shape in each form, and
 *   keeps the fastest.
 * oeb_batch_tuning_get: *count = the plan's launches; with record != NULL it also writes
 *   3 * count ints there (OEB_ERR_TOO_LARGE if capacity, in launches, is below count).
 * oeb_batch_tuning_apply: OEB_ERR_ARGUMENT if count differs from the plan's launches or a
 *   kb, shape or form is not one of the values above.  It records the step again for each
 *   (kb, shape) named, waits for the device to go idle, then swaps in the new tables.  On any error the
 *   plan is unchanged.  Results do not depend on the record.  Do not call it during a
 *   stream capture.
 * oeb_batch_signature: a 64-bit hash of the modes, each member's element size and domain
 *   (in order) and the launch count without fusion.  A record saved with one signature fits
 *   any plan with the same signature, in the same fusion grouping. */
/* Fusion grouping of a batch plan (OEB_FUSE_* as for oeb_set_fusion): which stages of the
 * chained step each member runs as one kernel.  oeb_batch_autotune tunes the launches of each
 * grouping, times a whole run of each, and keeps the faster grouping with its choices; a
 * tuning record fits the grouping it was taken with, so set that grouping before applying it.
 * oeb_batch_set_fusion records the step again with `mask` and the default choices (as at
 * creation), and rebuilds the one-launch tables if the plan has them; it waits for the device
 * to go idle.  OEB_ERR_ARGUMENT for unknown bits.  Results do not depend on the grouping. */
OEB_API oeb_status oeb_batch_set_fusion(oeb_batch_plan* plan, int mask);
OEB_API oeb_status oeb_batch_get_fusion(const oeb_batch_plan* plan, int* mask);
OEB_API oeb_status oeb_batch_tuning_get(const oeb_batch_plan* plan, int* record, int capacity, int* count);
OEB_API oeb_status oeb_batch_tuning_apply(oeb_batch_plan* plan, const int* record, int count);
OEB_API oeb_status oeb_batch_signature(const oeb_batch_plan* plan, uint64_t* out);
/* Kernel launches per run (one batched launch per recorded position and precision, or one
 * launch per member where the autotuner chose per-member launches), and interior points
 * per run (all members). */
OEB_API int oeb_batch_launches(const oeb_batch_plan* plan);
OEB_API int64_t oeb_batch_points(const oeb_batch_plan* plan);
/* Device bytes held by the plan (chain workspaces, scratch arena, tables). */
OEB_API size_t oeb_batch_plan_bytes(const oeb_batch_plan* plan);
OEB_API oeb_status oeb_batch_plan_destroy(oeb_batch_plan* plan);

/* The one-launch form (no counterpart in the reference).  With OEB_BATCH_FORM_ONE_LAUNCH a
 * run is ONE launch of a persistent step kernel (plus a memset of its counters) that runs
 * the whole step of every member, FP64 and FP32 alike: each member's recorded launches,
 * forward then adjoint, become its tasks, and a task waits on the device until every tile of
 * its member's previous task is done.  Members do not wait for each other.  The waits are
 * bounded: one that lasts longer than the plan's wait limit (2 s by default) sets the run's
 * status to OEB_ERR_TIMEOUT, after which every CTA stops at its next tile and the run's
 * outputs are incomplete.  Results are bit-identical to the per-launch form.
 * oeb_batch_set_form: form OEB_BATCH_FORM_PER_LAUNCH (the default) or _ONE_LAUNCH; kb is the
 *   k-blocking the one-launch tasks are recorded with (0 = each kernel's default, 1, 2, 4,
 *   8) and ctas_per_sm the build of the step kernel (2, 3 or 4 CTAs an SM: registers capped
 *   at 128, 80 or 64 a thread; 0 = 2); both ignored for the per-launch form.
 *   OEB_ERR_ARGUMENT for other values.  Building the one-launch tables records the step
 *   again and waits for the device to go idle; do not call it during a stream capture.
 * oeb_batch_get_form: the form, and kb and ctas_per_sm for the one-launch form (-1 for the
 *   other).
 * oeb_batch_autotune_form: times whole runs -- the per-launch form as the plan stands, then
 *   the one-launch form with each kb and each build -- keeps the fastest, and writes its
 *   time per run (ms) to *ms when ms is not NULL.
 * oeb_batch_step_waits: waits for the device to go idle, then reads the last one-launch
 *   run's waits that had to poll: their total time over all CTAs (us) and their number.
 * oeb_batch_step_status: waits for the device to go idle, then reads the status of the last
 *   one-launch run: 0, or OEB_ERR_TIMEOUT with *task (if not NULL) the task whose wait gave up.
 * oeb_batch_set_wait_limit: the longest one wait may last, in ns (> 0).
 * oeb_batch_withhold: a test of the bounded waits.  on != 0 makes the first task of the
 *   one-launch form wait for a count that nothing writes, so the next run ends with
 *   OEB_ERR_TIMEOUT after the wait limit; on == 0 restores it.  OEB_ERR_ARGUMENT before the
 *   one-launch tables exist. */
#define OEB_BATCH_FORM_PER_LAUNCH 0
#define OEB_BATCH_FORM_ONE_LAUNCH 1
OEB_API oeb_status oeb_batch_set_form(oeb_batch_plan* plan, int form, int kb, int ctas_per_sm);
OEB_API oeb_status oeb_batch_get_form(const oeb_batch_plan* plan, int* form, int* kb, int* ctas_per_sm);
OEB_API oeb_status oeb_batch_step_waits(oeb_batch_plan* plan, uint64_t* wait_us, uint64_t* waits);
OEB_API oeb_status oeb_batch_autotune_form(oeb_batch_plan* plan, void* stream, float* ms);
OEB_API oeb_status oeb_batch_step_status(oeb_batch_plan* plan, int* status, int* task);
OEB_API oeb_status oeb_batch_set_wait_limit(oeb_batch_plan* plan, uint64_t ns);
OEB_API oeb_status oeb_batch_withhold(oeb_batch_plan* plan, int on);
/* The one-launch form's ticket order, without a GPU (for tests and tools): for `members`
 * members with counts[m] tasks each and points[m] grid points, writes for every ticket t
 * (sum of counts entries) the task's member, its position in the member's sequence, and the
 * ticket of the task it waits for (its member's previous task; -1 for a member's first).
 * OEB_ERR_NULL for a NULL array, OEB_ERR_ARGUMENT for members < 1 or a negative count. */
OEB_API oeb_status oeb_batch_step_order(int members, const int* counts, const int64_t* points, int* member,
                                        int* position, int* dep);

/* ------------------------------------------------------------------------- */
/* CUDA graphs of library calls.  oeb_graph_begin starts capturing `stream`   */
/* (thread-local capture mode; not the legacy NULL stream); every library call */
/* made on it by this thread until oeb_graph_end is recorded, not run, and    */
/* oeb_graph_end instantiates the graph.  oeb_graph_launch replays it on any  */
/* stream.  The descriptors' pointers are baked in at capture, so a replay    */
/* reads and writes the same buffers.  Run each captured call once outside    */
/* capture first: one-time set-up (shared-memory limits, the scratch pool)   */
/* then happens before capture.  oeb_launch_count() counts the graph's       */
/* kernels at each launch, not at capture.                                   */
/* ------------------------------------------------------------------------- */
typedef struct oeb_graph oeb_graph;

OEB_API oeb_status oeb_graph_begin(void* stream);
OEB_API oeb_status oeb_graph_end(void* stream, oeb_graph** out);
OEB_API oeb_status oeb_graph_launch(oeb_graph* graph, void* stream);
OEB_API uint64_t oeb_graph_kernel_count(const oeb_graph* graph);
OEB_API oeb_status oeb_graph_destroy(oeb_graph* graph);

#ifdef __cplusplus
}
#endif

#endif /* OEB_GB300_H */
