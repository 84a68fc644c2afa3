/*
 * hydro_gb300.h -- C ABI of the GB300-native MaHyCo hydro hot path.
 *
 * Plain C types only (no C++ or torch types cross this boundary).  Every
 * call returns an int status: 0 = OK, < 0 = error; hydro_last_error() gives
 * the message of the last failure on the calling thread.
 *
 * What each entry point replaces in the reference (file:line within the
 * MaHyCo project):
 *   hydro_spec_default     option structs' defaults: includes/Options.h:9-21,
 *                          includes/GestionTemps.h:9-18, includes/Limiteurs.h
 *                          :10-25, includes/Eos.h:10-17, includes/CstMesh.h
 *   hydro_spec_parse_deck  LectureDonneesClass::LectureDonnees
 *                          (lecture_donnees/LectureDonnees.cc:12-226)
 *   hydro_run_create       scheme construction + set-up in main.cc:42-62 and
 *                          Vnr::simulate (vnr_remap/VnrRemap.cc:289-342) /
 *                          Eucclhyd::simulate (eucclhyd_remap/EucclhydRemap.cc
 *                          :233-286): mesh, initial state, dt_init
 *   hydro_run_step         Vnr::executeTimeLoopN (vnr_remap/VnrRemap.cc
 *                          :127-253) / Eucclhyd::executeTimeLoopN
 *                          (eucclhyd_remap/EucclhydRemap.cc:83-195), a bounded
 *                          number of cycles per call
 *   hydro_run_fetch        the arrays Vnr::dumpVariables /
 *                          Eucclhyd::dumpVariables hand to
 *                          PvdFileWriter2D::writeFile (VnrRemap.cc:255-287,
 *                          EucclhydRemap.cc:24-64), plus full state fields
 *   hydro_run_time         GestTemps t_n / deltat_n and the cycle counter n
 *   hydro_run_error        replaces the exit(1) aborts of the reference
 *                          (vnr_remap/PhaseRemapFinal.cc:174-196,
 *                          vnr_remap/PhaseLagrange.cc:358-369,
 *                          eucclhyd_remap/EucclhydRemap.cc:215-220)
 */
#ifndef HYDRO_GB300_H
#define HYDRO_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Scheme ids (includes/SchemaLagrange.h:10-15). */
#define HYDRO_SCHEME_EUCCLHYD 2000
#define HYDRO_SCHEME_VNR 2001

/* Limiter ids (includes/Limiteurs.h:10-25). */
#define HYDRO_LIM_MINMOD 300
#define HYDRO_LIM_SUPERBEE 301
#define HYDRO_LIM_VANLEER 302
#define HYDRO_LIM_MINMODG 1300
#define HYDRO_LIM_SUPERBEEG 1301
#define HYDRO_LIM_VANLEERG 1302
#define HYDRO_LIM_ARITHMETICG 1303
#define HYDRO_LIM_ULTRABEEG 1304

/* EOS ids (includes/Eos.h:10-14). */
#define HYDRO_EOS_VOID 100
#define HYDRO_EOS_PERFECT_GAS 101

/* Device error word bits (sticky per run). */
#define HYDRO_ERR_NAN 0x1u          /* NaN density/energy after remap       */
#define HYDRO_ERR_ENERGY 0x2u       /* |e_mat| > 5 in the VNR energy update */
#define HYDRO_ERR_DT_MIN 0x4u       /* dt < deltat_min (Eucclhyd)           */
#define HYDRO_ERR_NEGATIVE 0x8u     /* negative mass/energy zeroed (info)   */

/* Options of one hydro run.  Field meaning mirrors the reference's option
 * structs; hydro_spec_default() fills the reference defaults. */
typedef struct hydro_spec {
  int scheme;            /* HYDRO_SCHEME_*                                  */
  int test_case;         /* CasTest id (includes/CasTest.h:10-32)           */
  int nx, ny;            /* cells in x / y                                  */
  double dx, dy;         /* cell sizes (X_EDGE_LENGTH / Y_EDGE_LENGTH)      */
  int nbmat;             /* 1..3                                            */
  int eos[3];            /* HYDRO_EOS_* per material                        */
  double gamma[3];       /* Eos::gammap                                     */
  double gamma_scalar;   /* Eos::gamma (VNR pseudo-viscosity, init)         */
  double final_time;
  double output_time;
  double dt_init;        /* deck value; VNR with Lagrange recomputes it     */
  double dt_min;
  double cfl;            /* GestTemps::cfl (Eucclhyd; VNR hard-codes its own)*/
  long max_cycles;       /* stop after this many cycles; 0 = no cap         */
  int space_order;
  int projection;        /* AvecProjection                                  */
  int projection_conservative;
  int projection_order;  /* 1, 2 or 3                                       */
  double threshold;
  int limiter;           /* projectionLimiterId                             */
  int pb;                /* projectionAvecPlateauPente                      */
  int pb_mixte;          /* projectionLimiteurMixte                         */
  int limiter_pure;      /* projectionLimiterIdPure                         */
  int pb_complet;        /* projectionPlateauPenteComplet                   */
  int pseudo_centree;
  int dual_mass_flux;    /* methode_flux_masse: 0 A1, 1 A2, 2 PB            */
  int sans_lagrange;     /* advection cases: no Lagrange phase              */
  int init_variant;      /* 0 reference init; 1 bi-material Sod with a 50/50
                            mixed cell row/column at the interface          */
  double energy_limit;   /* VNR aborts when |e_mat| exceeds it (5 in the
                            reference, vnr_remap/PhaseLagrange.cc:358);
                            <= 0 disables the check                         */
} hydro_spec;

typedef struct hydro_ctx hydro_ctx;  /* device, streams, arena            */
typedef struct hydro_run hydro_run;  /* one mesh instance resident in HBM  */

const char* hydro_last_error(void);

int hydro_spec_default(hydro_spec* spec);
int hydro_spec_parse_deck(const char* path, hydro_spec* spec);

/* A context owns a stream on the device, the pinned staging (3 x 8 MiB) and
 * the host copy threads through which hydro_run_fetch hands fields over. */
int hydro_ctx_create(int device, size_t hbm_budget_bytes, hydro_ctx** out);
void hydro_ctx_destroy(hydro_ctx* ctx);

int hydro_run_create(hydro_ctx* ctx, const hydro_spec* spec, hydro_run** out);
/* Advance at most ncycles cycles (stops early at final_time / max_cycles);
 * *done is set to 1 once the reference loop condition ends the run. */
int hydro_run_step(hydro_run* run, int ncycles, int* done);
/* Copy a named field (see hydro_run_field_size) into host memory.  Besides
 * the full-state fields, the names the reference's dumpVariables gives its
 * output variables fetch exactly what it writes at the start of the next
 * cycle: "Pressure", "Density", "Energy", VNR "fracvol1", "fracvol2" (cell)
 * and "VitesseX", "VitesseY" (node), Eucclhyd "F1".."F3", "VelocityX",
 * "VelocityY" (vnr_remap/VnrRemap.cc:264-278, eucclhyd_remap/EucclhydRemap.cc
 * :43-50).  Returns once the values are in host_dst (any host memory); the
 * fetches of one context run one at a time. */
int hydro_run_fetch(hydro_run* run, const char* field, double* host_dst,
                    size_t n);
size_t hydro_run_field_size(hydro_run* run, const char* field);
int hydro_run_time(hydro_run* run, double* t, double* dt, long* cycle);
int hydro_run_error(hydro_run* run, unsigned* code, long* cell);
int hydro_run_destroy(hydro_run* run);

/* Output-driven stepping (the caller side of Vnr::dumpVariables,
 * vnr_remap/VnrRemap.cc:255-287, and Eucclhyd::dumpVariables,
 * eucclhyd_remap/EucclhydRemap.cc:24-64): advances at least one and at most
 * ncycles cycles and stops before the first later cycle whose start time
 * t_n satisfies t_n >= t_out || t_n == 0, the reference's dump condition with
 * t_out = lastDump + output_time.  *paused = 1 when it stopped there (the
 * caller writes its output, then calls again), *done = 1 when the run
 * ended.  The test runs on the device, so no cycle waits for the host. */
int hydro_run_step_to_output(hydro_run* run, int ncycles, double t_out,
                             int* done, int* paused);

/* Checkpoint / restart (no counterpart in the reference).  A checkpoint,
 * taken between cycles, holds the run's options and its whole device state
 * (fields, control block with time, dt, cycle count and error word); a
 * restored run continues bit for bit as the original.  Files are tied to the
 * library's memory layout (rejected otherwise) and carry a content hash
 * (truncated or corrupted files are rejected). */
int hydro_run_checkpoint(hydro_run* run, const char* path);
int hydro_run_restore(hydro_ctx* ctx, const char* path, hydro_run** out);

/* Asynchronous form of hydro_run_step: enqueue cycles on the context's
 * stream; hydro_run_sync waits and reports whether the run has ended. */
int hydro_run_enqueue(hydro_run* run, int ncycles);
int hydro_run_sync(hydro_run* run, int* done);
long long hydro_run_kernel_launches(hydro_run* run);
size_t hydro_run_device_bytes(hydro_run* run);
void* hydro_ctx_stream(hydro_ctx* ctx);

/* Measurement helpers (no counterpart in the reference). */
int hydro_run_timed(hydro_run* run, int ncycles, float* ms);
int hydro_run_profile(hydro_run* run, int ncycles, double* ms,
                      long long* launches, int nkinds);
const char* hydro_kernel_name(int kind);
int hydro_kernel_kinds(void);
int hydro_fp64_peak(int device, double* tflops);
/* The integer-pipe binary64 operations the kernels use for the common case
 * (normal operands and result): op 0 a*b, 1 a+b, 2 a/b, 3 sqrt(a), 4 a-b,
 * for n elements of device arrays a, b.  soft = the fast path's result,
 * hw = the FP64 instruction's, fast[i] = 1 where the fast path applies
 * (elsewhere the kernels use the FP64 instruction).  Asynchronous on
 * stream. */
int hydro_softfp_check(int op, const double* a, const double* b, double* soft, double* hw,
                       unsigned char* fast, long long n, void* stream);
/* Operations per second of dependent chains of mul, add, div, sqrt:
 * rates[2k] the FP64 instruction, rates[2k+1] the integer-pipe form. */
int hydro_softfp_rates(int device, double* rates);

/* Batched form (no counterpart in the reference, which advances one mesh
 * per scheme object; each run's cycle is Vnr::executeTimeLoopN's cycle).
 * Advances every run of the list by up to ncycles cycles with one
 * persistent launch per phase for all of them; runs that end stop
 * independently.  All runs must belong to ctx.  The first cycles of a new
 * list tune tile widths and grid sizes on the real work (results do not
 * depend on the tuning).  *nactive = runs still going. */
int hydro_batch_step(hydro_ctx* ctx, hydro_run* const* runs, int nruns,
                     int ncycles, int* nactive);
int hydro_batch_enqueue(hydro_ctx* ctx, hydro_run* const* runs, int nruns,
                        int ncycles);
int hydro_batch_timed(hydro_ctx* ctx, hydro_run* const* runs, int nruns,
                      int ncycles, float* ms);
int hydro_batch_profile(hydro_ctx* ctx, hydro_run* const* runs, int nruns,
                        int ncycles, double* ms, long long* launches,
                        int nkinds);
/* Tile width and height (items) and grid (blocks) chosen per batched phase
 * (nphases >= 13: VNR Lagrange nodes, cells, face gradients, slopes, faces,
 * update, dual slopes, dual update, final, then Eucclhyd cell pre-pass,
 * nodes, cells, final); returns 1 once a timed tuning pass has chosen
 * them. */
int hydro_batch_config(hydro_ctx* ctx, int* width, int* height, int* grid,
                       int nphases);
int hydro_batch_set_tuning(hydro_ctx* ctx, int enable);
long long hydro_batch_kernel_launches(hydro_ctx* ctx);

/* Serving (no counterpart in the reference): requests are hydro runs that
 * arrive at any time; a worker thread of the context admits them in arrival
 * order while the HBM budget (their arenas' bytes) and the slot limit allow,
 * advances every resident run together in batched ticks, and retires each run
 * at its own end.  Results equal the same run advanced alone. */
typedef struct hydro_serve_done {
  long req_id;
  int status;        /* device error word; -1 when the run could not start */
  double latency_s;  /* submission to retirement                          */
  long cycles;       /* cycles the run did                                */
  long cells;
  double wait_s;     /* submission to admission (HBM budget, slots)       */
  double resident_s; /* placement on the device to retirement             */
} hydro_serve_done;
typedef struct hydro_serve_stats {
  long submitted, admitted, completed, failed;
  long resident, waiting, peak_resident;
  long ticks, cycles;
  size_t bytes_in_use, peak_bytes;
  double cell_updates;  /* of completed runs                         */
  double busy_s;        /* first admission to last retirement        */
} hydro_serve_stats;
/* budget_bytes 0: the context's budget (0 there: none); other arguments
 * <= 0 keep the defaults (256 slots, ticks of up to 8 cycles, 4 host
 * threads preparing initial states). */
int hydro_serve_config(hydro_ctx* ctx, size_t budget_bytes, int max_resident,
                       int tick_cycles, int prep_threads);
/* keep = 1 holds the finished run for hydro_serve_result until
 * hydro_serve_release; keep = 0 frees it at retirement. */
int hydro_serve_submit(hydro_ctx* ctx, const hydro_spec* spec, int keep,
                       long* req_id);
/* 1: one completion popped into *out; 0: none within timeout_s. */
int hydro_serve_poll(hydro_ctx* ctx, double timeout_s, hydro_serve_done* out);
hydro_run* hydro_serve_result(hydro_ctx* ctx, long req_id);
int hydro_serve_release(hydro_ctx* ctx, long req_id);
int hydro_serve_stats_get(hydro_ctx* ctx, hydro_serve_stats* out);
/* drain = 1 waits for every submitted request to finish. */
int hydro_serve_stop(hydro_ctx* ctx, int drain);

/* CFL time step of a VNR state held in caller device memory, allocating
 * nothing (no counterpart in the reference; it restates the reduction of
 * Vnr::computeDeltaT with the remap on).  For callers that may not call
 * cudaMalloc/cudaFree because their own pool owns the device memory.  Inputs:
 * node velocity planes d_u, d_v ((nx+1)*(ny+1) each), cell sound speed d_c
 * (nx*ny), the current dt_n; output: one double at d_dt_out.  It models the
 * remapped run only: cfl 0.05 and the sub-volumes of the Euler mesh, whose
 * nodes sit at (dx*j, dy*i) from the origin as the reference's mesh
 * generator places them (a run without remap uses cfl 0.1 and its moved
 * sub-volumes, which this function does not take).  Its scratch is a fixed
 * 32 KiB device array inside the library, so at most 1,048,576 cells are
 * accepted (larger meshes return an error).  The first call on a device
 * looks up that array's address in the device's primary context (the one
 * the CUDA runtime uses) and keeps it for the life of the process: call it
 * with that context current, make the first call before any stream capture,
 * and do not call it after resetting the device.  Calls that overlap on the
 * GPU share the scratch and race. */
int hydro_vnr_dt_noalloc(int nx, int ny, double dx, double dy,
                         const double* d_u, const double* d_v,
                         const double* d_c, double dt_n, double* d_dt_out,
                         void* stream);

#ifdef __cplusplus
}
#endif
#endif /* HYDRO_GB300_H */
