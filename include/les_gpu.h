/*
 * les_gpu.h -- C-ABI of the GB300 (sm_103a) per-timestep solver of MPI-LES.
 *
 * The library keeps one urban domain (or a batch of domains) resident in GPU memory
 * and advances it with the reference's eight solver subroutines, in the step order
 * of src/main.f95:260-296 (velnw -> bondv1 -> velfg -> feedbf -> les -> adam -> press).
 * Each entry point below replaces one reference interface; the replaced Fortran
 * routine is cited beside it.  Plain C types only: no CUDA or torch types cross
 * this boundary, so Fortran (ISO_C_BINDING), C, C++ and Python (ctypes) can bind it.
 *
 * Conventions
 *   - Every function returns an int status: LES_OK (0) or a negative LES_ERR_* code.
 *     les_gpu_last_error() gives the message of the last failure on a handle.
 *   - Arrays cross the boundary in the reference's Fortran layout: column-major,
 *     i fastest, with the declared lower/upper bounds passed as lb[3]/ub[3]
 *     (for example u is (0:im+1,-1:jm+1,0:km+1), src/main.f95:147).  1-D arrays use
 *     lb[0]/ub[0] with lb[1]=ub[1]=lb[2]=ub[2]=0; 2-D arrays use lb[0..1]/ub[0..1].
 *   - Work is queued on the handle's own CUDA stream.  Calls on one handle must come
 *     from one host thread at a time.  les_gpu_download() and les_gpu_sync() are the
 *     synchronisation points (like the reads of src/module_LES_combined_ocl.f95:562-571).
 *   - There is no CPU fallback: without a usable GPU, les_gpu_create() fails with
 *     LES_ERR_CUDA.
 */
#ifndef LES_GPU_H
#define LES_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LES_GPU_ABI_VERSION 2

/* status codes */
#define LES_OK 0
#define LES_ERR_ARG (-1)      /* bad argument (size, extents, field id, value)      */
#define LES_ERR_CUDA (-2)     /* CUDA runtime error (message in last_error)         */
#define LES_ERR_STATE (-3)    /* call out of order (e.g. step before setup commit)  */
#define LES_ERR_NOMEM (-4)    /* device memory exhausted                            */
#define LES_ERR_NUMERIC (-5)  /* non-finite values detected by les_gpu_check_finite */
#define LES_ERR_BUSY (-6)     /* batch slot or request refused (capacity)           */
#define LES_ERR_IO (-7)       /* a file could not be opened, written or read        */

/* Field ids.  3-D state and work arrays (extents as declared in src/main.f95:63-159). */
enum les_field {
  LES_FIELD_U = 1,      /* (0:im+1,-1:jm+1, 0:km+1)  main.f95:147 */
  LES_FIELD_V = 2,      /* (0:im+1,-1:jm+1, 0:km+1)  main.f95:151 */
  LES_FIELD_W = 3,      /* (0:im+1,-1:jm+1,-1:km+1)  main.f95:153 */
  LES_FIELD_P = 4,      /* (0:im+2, 0:jm+2, 0:km+1)  main.f95:144 */
  LES_FIELD_F = 5,      /* (0:im, 0:jm, 0:km)        main.f95:120 */
  LES_FIELD_G = 6,
  LES_FIELD_H = 7,
  LES_FIELD_FOLD = 8,   /* (1:im, 1:jm, 1:km)        main.f95:124 */
  LES_FIELD_GOLD = 9,
  LES_FIELD_HOLD = 10,
  LES_FIELD_USUM = 11,  /* (0:im, 0:jm, 0:km)        main.f95:148 */
  LES_FIELD_VSUM = 12,
  LES_FIELD_WSUM = 13,
  LES_FIELD_RHS = 14,   /* (0:im+1, 0:jm+1, 0:km+1)  main.f95:145 */
  LES_FIELD_SM = 15,    /* (-1:im+1,-1:jm+1, 0:km+1) main.f95:146 */
  LES_FIELD_BMASK1 = 16,/* (-1:im+1, 0:jm+1, 0:km+1) values 0 or 1 */
  LES_FIELD_CMASK1 = 17,/* (0:im+1,-1:jm+1, 0:km+1)  values 0 or 1 */
  LES_FIELD_DMASK1 = 18,/* (0:im+1, 0:jm+1, 0:km+1)  values 0 or 1 */
  LES_FIELD_CN1 = 20,   /* (1:im, 1:jm, 1:km)        upload only (init.f95:98-104) */
  /* 1-D grid and Poisson coefficient arrays (grid.f95, init.f95:82-95) */
  LES_FIELD_DX1 = 32,   /* (-1:im+1) */
  LES_FIELD_DY1 = 33,   /* (0:jm+1)  */
  LES_FIELD_DZN = 34,   /* (-1:km+2) */
  LES_FIELD_DZS = 35,   /* (-1:km+2) */
  LES_FIELD_DXS = 36,   /* (0:im)    */
  LES_FIELD_DYS = 37,   /* (0:jm)    */
  LES_FIELD_Z2 = 38,    /* (0:km+2)  */
  LES_FIELD_CN2L = 39,  /* (1:im)    */
  LES_FIELD_CN2S = 40,
  LES_FIELD_CN3L = 41,  /* (1:jm)    */
  LES_FIELD_CN3S = 42,
  LES_FIELD_CN4L = 43,  /* (1:km)    */
  LES_FIELD_CN4S = 44,
  LES_FIELD_DELX1 = 45, /* (1:km) download only: les.f95:38-42 */
  /* 2-D inflow planes applied by bondv1 on i = 0, 1 (replace bondv1.f95:33-54) */
  LES_FIELD_UIN = 53,   /* (1:jm, 1:km) */
  LES_FIELD_VIN = 54,
  LES_FIELD_WIN = 55,
  /* time averages of les_gpu_aveflow (aveflow.f95:7-22), download only, available
   * after its first call */
  LES_FIELD_AVEU = 100,    /* (1:im, 1:jm, 0:km)   */
  LES_FIELD_AVEV = 101,    /* (1:im, 1:jm, 0:km)   */
  LES_FIELD_AVEW = 102,    /* (1:im+1, 1:jm, 0:km+2) */
  LES_FIELD_AVEP = 103,    /* (1:im, 1:jm, 1:km) for this one and the rest */
  LES_FIELD_AVEL = 104,
  LES_FIELD_AVEUU = 105,
  LES_FIELD_AVEVV = 106,
  LES_FIELD_AVEWW = 107,
  LES_FIELD_AVESM = 108,
  LES_FIELD_AVESMSM = 109,
  LES_FIELD_UWFX = 110
};

typedef struct les_dims {
  int im, jm, km;       /* interior cells; jm must be even for the fused SOR sweep */
} les_dims;

typedef struct les_params {
  float dt, ro, vn;     /* set.f95:89-92 (0.05, 1.1763, 15.83e-6)                */
  float alpha, beta;    /* IBM feedback gains, set.f95:94-95 (-10, -1)           */
  float omega, pjuge;   /* SOR relaxation and tolerance, press.f95:43-45         */
  int nmaxp;            /* SOR iteration cap, press.f95:44 (50)                  */
  int sor_fixed;        /* 1: always nmaxp iterations; 0: exit on sor < pjuge     */
  int sor_ksplit;       /* 0: split the SOR k-march into chunks when the domain's
                         * tiles leave SMs idle (a domain alone on the GPU); 1: never
                         * (domains that share the GPU; les_batch_add sets it)    */
} les_params;

/* Synthetic urban scenario (the configs' generator; replaces the GIS inputs read
 * by feedbfm.f95:52-77 and the fixed inflow of bondv1.f95:33-54). */
typedef struct les_scenario {
  int im, jm, km;
  float dx, dy;                 /* 4 m, grid.f95:36-69                              */
  int dz_law;                   /* 0: grid.f95:114-135 law; 1: geometric            */
  float dz0, dz_ratio;          /* geometric law: dzn(1) = dz0, dzn(k) = dzn(k-1)*r  */
  unsigned long long seed;
  float coverage;               /* building plan-area fraction (0 = no buildings)    */
  int fp_min, fp_max;           /* block footprint side, cells                       */
  float h_min, h_max;           /* block height, m                                   */
  int inflow_law;               /* 0: 5 m/s uniform (bondv1.f95:33-54); 1: power law */
  float u_ref, z_ref, pl_exp;   /* power law U(z) = u_ref*(z/z_ref)^pl_exp           */
  float direction_deg;          /* inflow direction, degrees                         */
  float noise;                  /* fixed uniform +-noise on inflow cells, m/s        */
} les_scenario;

typedef struct les_handle les_handle;

/* ---- host-side setup (run once per domain; no GPU needed) ---------------------- */

/* grid.f95:5-182 for runtime sizes.  Output arrays at their Fortran extents:
 * dx1(-1:im+1) dxl(0:im) dxs(0:im) dy1(0:jm+1) dyl(0:jm) dys(0:jm) dzn(-1:km+2)
 * dzs(-1:km+2) z2(0:km+2). */
int les_setup_grid(int im, int jm, int km, float dx, float dy, int dz_law, float dz0,
                   float dz_ratio, float *dx1, float *dxl, float *dxs, float *dy1, float *dyl,
                   float *dys, float *dzn, float *dzs, float *z2);
/* init.f95:82-107: cn2s,cn2l(1:im) cn3s,cn3l(1:jm) cn4s,cn4l(1:km) cn1(1:im,1:jm,1:km);
 * cn1 may be NULL. */
int les_setup_poisson(int im, int jm, int km, const float *dxs, const float *dys,
                      const float *dzs, float *cn2s, float *cn2l, float *cn3s, float *cn3l,
                      float *cn4s, float *cn4l, float *cn1);
/* feedbfm.f95:25-116 with zbm(1:im,1:jm) given: masks at their Fortran extents. */
int les_setup_masks(int im, int jm, int km, const float *zbm, const float *z2,
                    const float *dzn, float *amask1, float *bmask1, float *cmask1,
                    float *dmask1);
/* The interior volume sum(dx1(i)*dy1(j)*dzn(k)) that rhsav and pav divide by
 * (press.f95:65-72, 124-133): each product rounded to FP32, summed in FP64 in the
 * loop order k, j, i.  dx1(-1:im+1), dy1(0:jm+1), dzn(-1:km+2).  O(im + jm + km x
 * distinct (dx1, dy1) pairs) when the partial sums are provably exact in FP64 (then
 * every order gives the sequential sum's bits); else the sequential loop. */
int les_setup_area(int im, int jm, int km, const float *dx1, const float *dy1, const float *dzn,
                   double *area);
/* Seeded synthetic scenario: zbm(1:im,1:jm) heightmap and uin/vin/win(1:jm,1:km)
 * inflow planes.  Deterministic for a given seed on every host. */
int les_scenario_generate(const les_scenario *sc, float *zbm, float *uin, float *vin,
                          float *win);
/* Bytes of device memory one domain of this size needs (admission control). */
size_t les_domain_bytes(int im, int jm, int km);

/* ---- one resident domain ------------------------------------------------------- */

/* Allocate the device state of one domain, all fields zero (init.f95:46-69).
 * Replaces the buffer set-up of initialise_LES_kernel (module_LES_combined_ocl.f95:14). */
int les_gpu_create(const les_dims *dims, const les_params *params, les_handle **out);
int les_gpu_destroy(les_handle *h);
/* Copy a field between host (Fortran layout, extents lb..ub) and device. */
int les_gpu_upload(les_handle *h, int field, const float *host, const int lb[3],
                   const int ub[3]);
int les_gpu_download(les_handle *h, int field, float *host, const int lb[3],
                     const int ub[3]);
/* Asynchronous download of a 3-D field's box (no reference counterpart: it lets the
 * per-step output of main.f95:311-327 overlap the next step).  The box is snapshotted on
 * the device in stream order -- later steps may be queued at once and do not change
 * what is copied -- and copied to `host` on a copy stream of the handle.  *ticket
 * identifies the copy; les_gpu_download_wait(h, ticket) returns once it is in host
 * memory.  `host` must stay valid until then (pinned memory lets the copy overlap).
 * At most 8 copies are in flight per handle: a ninth call first waits for the oldest. */
int les_gpu_download_async(les_handle *h, int field, float *host, const int lb[3], const int ub[3],
                           long long *ticket);
int les_gpu_download_wait(les_handle *h, long long ticket);
/* Validate the uploaded grid/coefficients/masks/inflow and derive the per-domain
 * constants (les.f95:38-42 delx1, the log-law factor of vel2.f95:138).  Required
 * once before the first solver call and after any later grid upload. */
int les_gpu_commit_setup(les_handle *h);
/* feedbfm.f95:87-116 on the device: the b, c, d masks (1 inside a building, where
 * zbm(i,j) > z2(k) + 0.5*dzn(k), else 0; 0 in the halos) made from the heightmap
 * zbm(1:im,1:jm) (column-major, i fastest) in place of uploading the three 3-D mask
 * arrays.  Needs z2 and dzn uploaded first; masks uploaded later change the result
 * per field as before.  Synchronises the handle's stream. */
int les_gpu_feedbfm(les_handle *h, const float *zbm);
/* Convenience: generate the scenario, run the host setup and upload + commit. */
int les_gpu_setup_scenario(les_handle *h, const les_scenario *sc);

/* The eight solver subroutines, on device-resident state. */
int les_gpu_velnw(les_handle *h);                    /* velnw.f95:5   */
int les_gpu_bondv1(les_handle *h, int n);            /* bondv1.f95:5  */
int les_gpu_velfg(les_handle *h);                    /* velFG.f95:6 (vel2 fused)   */
int les_gpu_feedbf(les_handle *h);                   /* feedbf.f95:5  */
int les_gpu_les(les_handle *h);                      /* les.f95:6 (boundsm fused)  */
int les_gpu_adam(les_handle *h);                     /* adam.f95:5    */
int les_gpu_press(les_handle *h, int n, int nmax);   /* press.f95:9   */
int les_gpu_bondfg(les_handle *h);                   /* bondFG.f95:5  */
int les_gpu_boundp1(les_handle *h);                  /* boundp.f95:28 */
int les_gpu_boundp2(les_handle *h);                  /* boundp.f95:7  */

/* One whole time step n (velnw .. press) through the fused kernels, launched as a
 * captured CUDA graph.  Mirrors run_LES_kernel(n, nmax), main.f95:251. */
int les_gpu_step(les_handle *h, int n, int nmax);
/* Steps n0 .. n0+nsteps-1 back to back (the main.f95:247 loop body). */
int les_gpu_run(les_handle *h, int n0, int nsteps, int nmax);
/* Waits for the handle's stream.  LES_ERR_STATE if a kernel since the last sync gave
 * up a bounded wait for its own copies (never expected; the results of that work are
 * void, and the flag is cleared). */
int les_gpu_sync(les_handle *h);
/* Diagnostics of the last press call: out[0] SOR iterations, out[1] last residual
 * sum (FP64), out[2] uout, out[3] rhsav, out[4] pav.  Synchronises. */
int les_gpu_diag(les_handle *h, double out[5]);
/* Sets *bad to the number of non-finite interior values of u, v, w, p. */
int les_gpu_check_finite(les_handle *h, long long *bad);
/* The handle's CUDA stream (a cudaStream_t), for callers that time or overlap work. */
int les_gpu_stream(les_handle *h, void **stream);
/* Volume-weighted interior mean of a 3-D field, sum(x*dx1*dy1*dzn)/sum(dx1*dy1*dzn)
 * over i=1..im, j=1..jm, k=1..km, in the order and FP32 rounding press uses for pav
 * (press.f95:124-133); the field is not changed.  No counterpart in the reference:
 * an addition for callers that must not allocate device memory when they call (a
 * pre-sized memory cap, a host allocator that owns the device, a monitor between
 * steps).  It allocates nothing: its scratch is one static device array per device,
 * shared by all calls, which keeps what the last call left (each call clears what must
 * start at zero).  Calls that overlap in time race on it.  The array's address is
 * looked up on the first call from a device: make that call outside stream capture.
 * Domains with more than LES_NOALLOC_MAX_PARTS reduction blocks of 64 x 4 x 16 cells
 * ((im+63)/64 * (jm+3)/4 * ((km+15)/16); 600x600x90 has 9000) are refused with
 * LES_ERR_ARG.  Synchronises the handle's stream. */
#define LES_NOALLOC_MAX_PARTS 65536 /* 512 KiB of FP64 block partials */
int les_gpu_field_mean_noalloc(les_handle *h, int field, double *mean);
/* Kernel launches issued on this handle since creation (all stages). */
long long les_gpu_launch_count(les_handle *h);
int les_gpu_last_error(les_handle *h, char *buf, size_t len);

/* ---- batches of resident domains (ensembles, continuous batching) ---------------
 * A batch holds caller-owned domain handles and a step counter per member.
 * les_batch_step enqueues one time step (n, nmax) of every member whose n <= nmax,
 * each on the member's own stream, without host synchronisation, and advances n; the
 * members' kernels overlap on the GPU.  Members join and leave between steps.  A
 * member's arithmetic never depends on the others: its result is the same alone and
 * in any mix.  Calls on one batch are serialised internally.  Cross-stream overlap
 * is bounded by CUDA_DEVICE_MAX_CONNECTIONS (set it, up to 32, before CUDA starts). */
typedef struct les_batch les_batch;
int les_batch_create(les_batch **out);
int les_batch_destroy(les_batch *b);  /* syncs members; does not destroy their handles */
/* *ok = 1 if the device's free memory holds one more domain of these dims plus
 * reserve_bytes (admission by free HBM; les_domain_bytes is the footprint). */
int les_batch_admit(const les_dims *dims, size_t reserve_bytes, int *ok);
/* Add a committed handle whose next step is n0 (1 for a fresh domain), run to nmax. */
int les_batch_add(les_batch *b, les_handle *h, int n0, int nmax, int *slot);
int les_batch_remove(les_batch *b, int slot);  /* syncs the member first */
/* One step of every unfinished member; *nlive = members with steps left after it.
 * By default each member's whole-step graph runs on its own stream.  With
 * les_batch_set_sor_launch(b, 1), each member's step runs up to its first SOR iteration
 * on its own stream; SOR iterations 2..nmaxp of all members (of one tile shape) then
 * run as one persistent launch over a work-list of every member's tiles, whose CTAs
 * wait (bounded) for a member's previous iteration before its next; the rest of each
 * step follows on the member's stream (members without a fused SOR sweep step alone).
 * Either way a member's fields are bitwise those of the domain stepped alone. */
int les_batch_step(les_batch *b, int *nlive);
/* persistent = 1: the persistent SOR launch over all members' tiles; 0 (default): each
 * member's whole-step graph on its own stream.  No counterpart in the reference. */
int les_batch_set_sor_launch(les_batch *b, int persistent);
/* Waits for every member; fails with LES_ERR_STATE if a dependency wait of a batched
 * SOR launch gave up since the last call (the members' SOR of that step is incomplete),
 * or if a member's own kernel gave up a bounded wait (as les_gpu_sync reports it). */
int les_batch_sync(les_batch *b);
/* Bound of the batched SOR launch's dependency waits, in polls of about 128 ns (default
 * 2^23, about a second).  hold_slot >= 0 makes that member's wait impossible, so that a
 * test can exercise the give-up path; -1 restores normal stepping.  No counterpart in
 * the reference. */
int les_batch_set_wait_limit(les_batch *b, long long polls, int hold_slot);
/* *n = the member's next step index (> nmax once finished). */
int les_batch_slot(les_batch *b, int slot, int *n, int *nmax);
int les_batch_last_error(les_batch *b, char *buf, size_t len);

/* aveflow(n,n1,...,nmax) of aveflow.f95:5-200, called after each step as main.f95:320
 * does: from step n1 on the time averages (LES_FIELD_AVEU..UWFX) accumulate v, p, u, w,
 * the squares of u, v, w, sm, sm and the u-w flux; at n == nmax they are divided by
 * nmax-n1+1 and the rms fluctuations and the mean-removed flux formed.  The averaging
 * arrays (11 fields) are allocated on the first call.  The reference's unformatted
 * writes of the averages at nmax are les_gpu_write_data10/11. */
int les_gpu_aveflow(les_handle *h, int n, int n1, int nmax);

/* ---- the reference's result and restart files ----------------------------------
 * gfortran unformatted sequential files, one record per Fortran write, each 3-D record
 * the interior box (1:im,1:jm,1:km), i fastest.  Big-endian markers and values, as the
 * reference is built (SConstruct:77, -fconvert=big-endian), unless flags has
 * LES_IO_LITTLE_ENDIAN.  Records over 2147483639 bytes are split into gfortran
 * subrecords (LES_IO_MAX_SUBRECORD in the environment lowers that limit, like
 * -fmax-subrecord-length).  The writers download the fields (they synchronise the
 * handle's stream); the reader uploads them.  The reference writes data20 and data21
 * when mod(n,1000) == 0 or n == nmax (press.f95:197, adam.f95:21): the caller keeps
 * that test around les_gpu_write_data20/21. */
#define LES_IO_LITTLE_ENDIAN 1
/* press.f95:205-216: u, v, w, p, usum, vsum, wsum */
int les_gpu_write_data20(les_handle *h, const char *path, int flags);
/* adam.f95:20-27: fold, gold, hold, fghold (never assigned in the reference: zeros) */
int les_gpu_write_data21(les_handle *h, const char *path, int flags);
/* anime.f95:370-490: the record (n, time) as int32 and real(4), then u, v, w, p, usum,
 * vsum, wsum */
int les_gpu_write_data30(les_handle *h, const char *path, int n, float time, int flags);
/* anime.f95:492-595: f, g, h, fold, gold, hold */
int les_gpu_write_data31(les_handle *h, const char *path, int flags);
/* aveflow.f95:209-263 (n == nmax): aveu, avew, avev -- in that order */
int les_gpu_write_data10(les_handle *h, const char *path, int flags);
/* aveflow.f95:273-344 (n == nmax): aveuu, aveww, avevv (the rms values), uwfx */
int les_gpu_write_data11(les_handle *h, const char *path, int flags);
/* ifdata_out(n,n0,n1,nmax,time,...) of anime.f95:326, called after every step
 * (main.f95:318): when n == n1-1 or n == nmax it writes <dir>/data30NNNNNN.dat and
 * <dir>/data31NNNNNN.dat (NNNNNN = n as i6.6) and sets *written (may be NULL) to 1;
 * otherwise it writes nothing and sets it to 0. */
int les_gpu_ifdata_out(les_handle *h, const char *dir, int n, int n1, int nmax, float time, int flags,
                       int *written);
/* The restart read of ifdata (ifdata.f95:252-480, ical == 1): n and time from data30's
 * first record, then the interiors (1:im,1:jm,1:km) of u, v, w, p, usum, vsum, wsum from
 * data30 and of f, g, h, fold, gold, hold from data31; halos keep their values.  Either
 * byte order is read.  A record shorter than im*jm*km values fails with LES_ERR_IO. */
int les_gpu_read_restart(les_handle *h, const char *data30, const char *data31, int *n, float *time);

/* Tile shape of press's fused SOR sweep.  nx: float4 columns per tile row, 32 (120
 * interior i cells) or 16 (56 cells, uniform cn1 only); ny: tile rows, 16/20/24/28
 * (and 32 with depth 2); kchunk: k planes per CTA (the march is split in k chunks when
 * kchunk < km); depth: SOR iterations per k-march, 1, or 2 (iteration l+1 trailing l by
 * two planes in the same march, so p and rhs cross HBM once per two iterations; 32
 * columns, ny 24/28/32, the whole march, omega = 1 and uniform x/y coefficients, else
 * the sweep runs depth 1).  The interior j rows of a tile are ny - 4 depth.  0 leaves a
 * value to the automatic choice.  The shape never changes the fields, only the speed
 * and the residual's summation order; with the exit on sor < pjuge (press.f95:119-121)
 * a two-iteration launch whose first iteration met the test is cut back to it.
 * les_gpu_set_sor_shape drops captured step graphs (the next step captures again);
 * les_gpu_sor_shape reports {nx, ny, kchunk, depth} in use, zeros for the
 * per-subroutine SOR (odd jm or km >= 511).  No reference counterpart: these are the
 * tuning knobs. */
int les_gpu_set_sor_shape(les_handle *h, int nx, int ny, int kchunk, int depth);
int les_gpu_sor_shape(les_handle *h, int out[4]);

/* Autotuner of the SOR tile shape and fusion depth per size class (im, jm, km, and the
 * device).  It times the candidate shapes on scratch copies of this domain's SOR
 * buffers: with shared = 0 the domain alone on the GPU (tile heights x k chunks, and
 * two-iteration marches), with shared = 1 many replicas running at once, the way batch
 * members share the GPU (16- and 32-column tiles, and two-iteration marches).  The fastest shape goes into a process-wide table that domains
 * of the class use from their next step on (les_batch_add marks a member shared);
 * les_gpu_set_sor_shape still overrides it.  Run it while nothing else uses the GPU.
 * out (or NULL): the shape chosen {nx, ny, kchunk, depth}, zeros when the domain has
 * no fused sweep;
 * us (or NULL): its microseconds per SOR iteration and domain; report (or NULL): the
 * candidates' timings as text, truncated to len bytes.
 * les_sor_tuned reads the table (1: found, 0: not tuned); les_sor_set_tuned writes an
 * entry (e.g. from a saved table), nx = 0 erases it. */
int les_gpu_tune_sor(les_handle *h, int shared, int out[4], double *us, char *report, size_t len);
int les_sor_tuned(int im, int jm, int km, int shared, int device, int out[4]);
int les_sor_set_tuned(int im, int jm, int km, int shared, int device, int nx, int ny, int kchunk, int depth);

/* Profiling: queue `reps` back-to-back launches of one stage on the handle's stream,
 * bracketed by CUDA events, and return the average milliseconds per repetition.
 * The stage really runs (it advances the state).  what: LES_PROF_*. */
enum les_prof {
  LES_PROF_SOR = 0,    /* one SOR iteration of press, as the whole step runs it */
  LES_PROF_VELFG = 1,  /* velfg (+ feedbf when fused in the step)                */
  LES_PROF_LES = 2,    /* les: eddy viscosity and viscous terms (+ adam fused)   */
  LES_PROF_VELNW = 3,
  LES_PROF_STEP = 4,   /* one whole step (n > 1)                                 */
  LES_PROF_SOR_SWEEP = 5 /* the fused SOR sweep kernel alone: per launch, events
                          * around sweeps 2..nmaxp of passes run as the step runs
                          * them (the first sweep reads p, a different kernel)     */
};
int les_gpu_profile(les_handle *h, int what, int reps, double *ms_avg);

#ifdef __cplusplus
}
#endif
#endif /* LES_GPU_H */
