/*
 * pars_gpu.h — C ABI of the GB300 (sm_103a) particle-tracing library
 * (libpars_gpu.so).
 *
 * The library replaces the CPU/TBB stages of the pars hot path behind plain C
 * calls: plain pointers and sizes, int32 status codes, no exceptions and no C++
 * or torch types.  Every function returns PARS_OK (0) or a negative status;
 * pars_gpu_last_error() gives the message of the last failure on a context.
 *
 * Units and conventions are the reference's: positions are pa::vector4
 * (x, y, z, w) FP32, fields are pa::vector_field (offset, size, spacing, data
 * [X][Y][Z] of xyz FP32 in C order), curves are the integral_curves buffers of
 * pa/include/pa/math/integral_curves.hpp:11-20 (vector4 vertices with the
 * termination vertex (-2,-2,-2,0) ending each curve, vector4 colours, int32
 * line indices), split into batches exactly as particle_tracer::
 * compute_round_info does (particle_tracer.cpp:210-234).
 *
 * Threading: calls on one context are serialised by the context; separate
 * contexts are independent.  Work is issued on the context's CUDA stream
 * (its own, or one set with pars_gpu_set_stream).  On its own stream a call's
 * work starts after the work already submitted to the legacy default stream;
 * callers that produce device inputs on another stream synchronise it first
 * or pass it with pars_gpu_set_stream.  Uploads return once their copy is
 * done, so the caller's buffer may be reused at once.
 */
#ifndef PARS_GPU_H
#define PARS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PARS_GPU_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------- */
enum pars_gpu_status
{
  PARS_OK                    =  0,
  PARS_ERR_INVALID_ARGUMENT  = -1,
  PARS_ERR_CUDA              = -2,
  PARS_ERR_OUT_OF_MEMORY     = -3,
  PARS_ERR_UNSUPPORTED       = -4,
  PARS_ERR_NOT_FOUND         = -5,
  PARS_ERR_BUDGET            = -6,
  PARS_ERR_CANCELLED         = -7,
  PARS_ERR_TIMEOUT           = -8,
  PARS_ERR_STATE             = -9
};

/* ---- enumerations ---------------------------------------------------------- */
/* Order of pa::variant_integrator (pa/include/pa/math/integrators.hpp:24-32). */
enum pars_integrator
{
  PARS_EULER                         = 0,
  PARS_MODIFIED_MIDPOINT             = 1,
  PARS_RUNGE_KUTTA_4                 = 2,
  PARS_RUNGE_KUTTA_CASH_KARP_54      = 3,
  PARS_RUNGE_KUTTA_DORMAND_PRINCE_5  = 4,
  PARS_RUNGE_KUTTA_FEHLBERG_78       = 5,
  PARS_ADAMS_BASHFORTH_2             = 6,
  PARS_ADAMS_BASHFORTH_MOULTON_2     = 7
};

/* How the integrator's stages see the field.
 * FROZEN:    the reference's behaviour — the right-hand side returns the
 *            velocity sampled once at the step start for every stage
 *            (particle_tracer.cpp:315-318), with the reference's FP32 operation
 *            order (bit-exact with the reference on equal inputs).
 * RESAMPLED: each stage samples the field at its own stage point (classical
 *            RK4: four samples per step).  Stage points outside the grid use
 *            the nearest boundary cell with its weight clamped to 0 or 1. */
enum pars_stage_mode
{
  PARS_STAGES_FROZEN    = 0,
  PARS_STAGES_RESAMPLED = 1
};

/* Order of pa::color_generator::mode (pa/include/pa/stages/color_generator.hpp:13-20). */
enum pars_color_mode
{
  PARS_COLOR_NONE           = -1,
  PARS_COLOR_HSL_CONSTANT_S =  0,
  PARS_COLOR_HSL_CONSTANT_L =  1,
  PARS_COLOR_HSV_CONSTANT_S =  2,
  PARS_COLOR_HSV_CONSTANT_V =  3,
  PARS_COLOR_RGB            =  4
};

/* pa::ftle_map_generator::mode (pa/include/pa/stages/ftle_map_generator.hpp:15-19). */
enum pars_ftle_mode
{
  PARS_FTLE_REGULAR               = 0,
  PARS_FTLE_FRACTIONAL_ANISOTROPY = 1
};

/* ---- types ------------------------------------------------------------------ */
/* Byte layout of pa::particle (pa/include/pa/math/particle.hpp:12-36): Eigen
 * Vector4f position (16-byte aligned), remaining_iterations,
 * vector_field_index (-1 = local block, 0..5 = neighbour face), original_rank,
 * Eigen Vector3i original_voxel; 48 bytes with the tail padding. */
typedef struct pars_particle
{
  float   position[4];
  int32_t remaining_iterations;
  int32_t vector_field_index;
  int32_t original_rank;
  int32_t original_voxel[3];
  int32_t padding[2];
} pars_particle;

/* The layout checks (offsets as in pa::particle with Eigen's 16-byte
 * Vector4f, particle.hpp:30-35). */
#ifdef __cplusplus
static_assert(sizeof(pars_particle) == 48, "pars_particle is 48 bytes like pa::particle");
static_assert(offsetof(pars_particle, position) == 0, "position at offset 0");
static_assert(offsetof(pars_particle, remaining_iterations) == 16, "remaining_iterations at offset 16");
static_assert(offsetof(pars_particle, vector_field_index) == 20, "vector_field_index at offset 20");
static_assert(offsetof(pars_particle, original_rank) == 24, "original_rank at offset 24");
static_assert(offsetof(pars_particle, original_voxel) == 28, "original_voxel at offset 28");
#else
_Static_assert(sizeof(pars_particle) == 48, "pars_particle is 48 bytes like pa::particle");
_Static_assert(offsetof(pars_particle, position) == 0, "position at offset 0");
_Static_assert(offsetof(pars_particle, remaining_iterations) == 16, "remaining_iterations at offset 16");
_Static_assert(offsetof(pars_particle, vector_field_index) == 20, "vector_field_index at offset 20");
_Static_assert(offsetof(pars_particle, original_rank) == 24, "original_rank at offset 24");
_Static_assert(offsetof(pars_particle, original_voxel) == 28, "original_voxel at offset 28");
#endif

/* partitioner::set_domain_size / rank_info (pa/source/stages/partitioner.cpp:8-53). */
typedef struct pars_partition_info
{
  int32_t grid_size[3];
  int32_t block_size[3];
  int32_t multi_rank[3];
  int32_t offset[3];              /* voxel offset of the block */
  int32_t ghosted_block_size[3];  /* +1 on the + side of interior faces */
  int32_t neighbor_rank[6];       /* faces -x,+x,-y,+y,-z,+z; -1 where absent */
} pars_partition_info;

/* Summary of one tracing call. */
typedef struct pars_gpu_trace_summary
{
  int64_t batches;        /* integral_curves batches produced */
  int64_t vertices;       /* vertices over all batches (after prune) */
  int64_t steps;          /* integrator steps taken (particle-steps) */
  int32_t rounds;         /* tracing rounds (1 for a single block) */
  int32_t padding;
} pars_gpu_trace_summary;

typedef struct pars_gpu_context pars_gpu_context;

/* ---- context ------------------------------------------------------------------ */
/* Creates a context on CUDA device `device` with its own non-blocking stream. */
int32_t     pars_gpu_create       (pars_gpu_context** context, int32_t device);
int32_t     pars_gpu_destroy      (pars_gpu_context*  context);
const char* pars_gpu_last_error   (const pars_gpu_context* context);
int32_t     pars_gpu_abi_version  (void);
/* Issues all later work on `stream` (a cudaStream_t); NULL restores the
 * context's own stream. */
int32_t     pars_gpu_set_stream   (pars_gpu_context* context, void* stream);
int32_t     pars_gpu_synchronize  (pars_gpu_context* context);
/* Device bytes currently held by the context. */
int32_t     pars_gpu_memory_in_use(pars_gpu_context* context, int64_t* bytes);

/* ---- vector_field (pa/include/pa/math/vector_field.hpp:14-24) ----------------- */
/* Uploads a field from HOST memory: xyz is [shape0][shape1][shape2][3] FP32
 * (the layout data_io.cpp:99-106 fills).  The device copy is padded to float4.
 * Every shape entry must be >= 2.  *field receives a handle. */
int32_t pars_gpu_field_upload       (pars_gpu_context* context, const float* xyz, const int32_t shape[3],
                                     const float offset[3], const float size[3], const float spacing[3], int32_t* field);
/* Same, from DEVICE memory (xyz already resident, e.g. produced on the GPU). */
int32_t pars_gpu_field_upload_device(pars_gpu_context* context, const float* device_xyz, const int32_t shape[3],
                                     const float offset[3], const float size[3], const float spacing[3], int32_t* field);
int32_t pars_gpu_field_release      (pars_gpu_context* context, int32_t field);
/* Shape, offset, size and spacing of a resident field (any pointer may be NULL). */
int32_t pars_gpu_field_info         (pars_gpu_context* context, int32_t field, int32_t shape[3], float offset[3],
                                     float size[3], float spacing[3]);
/* Copies a resident field (e.g. a flow map) to HOST xyz, [X][Y][Z][3] FP32. */
int32_t pars_gpu_field_download     (pars_gpu_context* context, int32_t field, float* xyz);
/* vector_field::contains + ::interpolate (vector_field.cpp:12-48) at n host
 * positions (vector4); velocity is 0 where the position is outside. */
int32_t pars_gpu_field_sample       (pars_gpu_context* context, int32_t field, const float* positions, int64_t n,
                                     uint8_t* inside, float* velocity);

/* ---- seed_generator::generate (pa/source/stages/seed_generator.cpp:9-21) ------- */
/* Writes up to `capacity` particles to host `particles` (may be NULL to count). */
int32_t pars_gpu_seed_generate(pars_gpu_context* context, const float offset[3], const float size[3], const float stride[3],
                               int32_t iterations, int32_t rank, pars_particle* particles, int64_t capacity, int64_t* count);

/* ---- partitioner (pa/source/stages/partitioner.cpp:8-53) ------------------------ */
int32_t pars_gpu_partition(int32_t ranks, int32_t rank, const int32_t domain_size[3], pars_partition_info* info);

/* ---- particle_tracer (pa/source/stages/particle_tracer.cpp:39-56, 210-337, 402-409)
 * Traces host particles through one block (`field`, no neighbours: particles
 * leaving it are dropped) and prunes, leaving the curves on the device.
 * integrator: any pars_integrator (integrators.hpp:16-23), with the
 * reference's frozen stages (PARS_STAGES_FROZEN) or re-sampled ones
 * (PARS_STAGES_RESAMPLED: each stage samples the field where it falls --
 * modified midpoint as Gragg's two substeps, Cash-Karp 5(4) and
 * Dormand-Prince 5 with 5th-order weights, Fehlberg 7(8) with 8th-order
 * weights, two-step Adams-Bashforth(-Moulton) after an RK4 first step). */
int32_t pars_gpu_trace(pars_gpu_context* context, int32_t field, const pars_particle* particles, int64_t count,
                       int32_t integrator, int32_t stage_mode, float step_size, pars_gpu_trace_summary* summary);
/* Same with the particles already in DEVICE memory. */
int32_t pars_gpu_trace_device(pars_gpu_context* context, int32_t field, const pars_particle* device_particles, int64_t count,
                              int32_t integrator, int32_t stage_mode, float step_size, pars_gpu_trace_summary* summary);

/* Partitioned domain on one GPU: the domain field (HOST, [X][Y][Z][3]) is split
 * into `ranks` blocks exactly as partitioner::set_domain_size does, each block
 * resident with its + side ghost layer; offset = voxel offset * spacing,
 * size = block_size * spacing (data_io.cpp:91-115).  *domain receives a handle. */
int32_t pars_gpu_domain_create (pars_gpu_context* context, const float* xyz, const int32_t domain_size[3],
                                const float spacing[3], int32_t ranks, int32_t* domain);
/* Same, from a DEVICE copy of the domain field. */
int32_t pars_gpu_domain_create_device(pars_gpu_context* context, const float* device_xyz, const int32_t domain_size[3],
                                      const float spacing[3], int32_t ranks, int32_t* domain);
int32_t pars_gpu_domain_release(pars_gpu_context* context, int32_t domain);
/* Traces seeds over a partitioned domain: rank r's seeds are
 * particles[seed_offsets[r] .. seed_offsets[r+1]).  Every round each block
 * traces its particles; particles leaving a block move to the face neighbour
 * through device queues (particle_tracer.cpp:280-309, 376-393), until none is
 * left.  The next round's particles of a block are, in order of the sending
 * block, the particles each sender handed over, in the sender's order. */
int32_t pars_gpu_trace_domain(pars_gpu_context* context, int32_t domain, const pars_particle* particles,
                              const int64_t* seed_offsets, int32_t integrator, int32_t stage_mode, float step_size,
                              pars_gpu_trace_summary* summary);

/* ---- round-by-round tracing: the stage calls of pipeline::execute's round loop
 * (pars/source/pipeline.cpp:153-209) on one GPU.  Every rank of the
 * partitioned domain is a block resident in this context; one call traces one
 * round of all of them at once.
 *
 * pars_gpu_domain_assemble: a domain whose blocks are fields the ranks
 * uploaded themselves (each rank's local_vector_field_, data_io.cpp:90-114):
 * the partitioner's grid of `ranks` blocks over domain_size (voxels), with
 * fields[r] = rank r's ghosted block (shape = its ghosted_block_size).  It
 * replaces particle_tracer::set_local_vector_field / set_neighbor_vector_fields
 * (pa/include/pa/stages/particle_tracer.hpp:44-45): on one GPU a block's face
 * neighbours are the other ranks' resident blocks.  Releasing the domain
 * leaves the fields to their owner. */
int32_t pars_gpu_domain_assemble(pars_gpu_context* context, int32_t ranks, const int32_t domain_size[3], const int32_t* fields,
                                 int32_t* domain);
/* One round of particle_tracer's sub-methods for every rank
 * (particle_tracer.cpp:210-393: compute_round_info, allocate, initialize,
 * trace, out_of_bounds_distribute), replacing particle_tracer.hpp:51-59.
 * Rank r's particles of this round are particles[offsets[r] .. offsets[r+1])
 * (HOST), or, with particles = NULL, the particles the previous round left on
 * the device for round `round`.  The round's curves, pruned, in
 * compute_round_info's batches per rank and tagged (rank, round), are appended
 * to the context's curves (round 0 starts them afresh).  Particles that left
 * their block through a face with a neighbour become the neighbour's particles
 * of the next round, ordered by sending rank, then by the sender's order;
 * next_offsets (HOST, ranks + 1 entries, may be NULL) receives each rank's
 * next-round count (all zero: check_completion holds).  summary: this round's
 * batches, vertices and steps. */
int32_t pars_gpu_round_trace(pars_gpu_context* context, int32_t domain, int32_t round, const pars_particle* particles,
                             const int64_t* offsets, int32_t integrator, int32_t stage_mode, float step_size,
                             int64_t* next_offsets, pars_gpu_trace_summary* summary);
/* Copies the next round's particles left by the last pars_gpu_round_trace to
 * HOST `particles` (next_offsets[ranks] of them, grouped by rank). */
int32_t pars_gpu_round_particles(pars_gpu_context* context, pars_particle* particles);

/* Curves of the last trace call, resident on the device.
 * pars_gpu_curves_index: index_generator::generate on every batch.
 * pars_gpu_curves_color: color_generator::generate on every batch (needs indices). */
int32_t pars_gpu_curves_index     (pars_gpu_context* context);
int32_t pars_gpu_curves_color     (pars_gpu_context* context, int32_t mode, float parameter);
int32_t pars_gpu_curves_batch_info(pars_gpu_context* context, int64_t batch, int64_t* vertices, int64_t* indices,
                                   int32_t* rank, int32_t* round);
/* Copies one batch to HOST memory; any pointer may be NULL. */
int32_t pars_gpu_curves_download  (pars_gpu_context* context, int64_t batch, float* vertices, float* colors, int32_t* indices);

/* ---- index / colour stages on host buffers -------------------------------------- */
/* index_generator::generate (index_generator.cpp:10-24) on one batch of n host
 * vertices; indices needs room for n entries. */
int32_t pars_gpu_index_generate(pars_gpu_context* context, const float* vertices, int64_t n, int32_t* indices, int64_t* index_count);
/* color_generator::generate (color_generator.cpp:16-39); colours the reference
 * leaves unwritten are left unchanged in `colors`. */
int32_t pars_gpu_color_generate(pars_gpu_context* context, const float* vertices, int64_t n, const int32_t* indices,
                                int64_t index_count, int32_t mode, float parameter, float* colors);

/* ---- flow map + FTLE ---------------------------------------------------------- */
/* flow_map_generator::generate (flow_map_generator.cpp:12-52) on one block:
 * one particle per voxel of an int(shape * scale) grid with spacing
 * spacing / scale, advected with particle_advector's rules
 * (particle_advector.cpp:74-139; at most iterations - 1 steps).  The flow map
 * becomes a new field handle (*flow_map) resident on the device (re-sampled
 * stages also keep the positions' sub-ulp residuals, as for batched jobs
 * below).  Integrators as for pars_gpu_trace. */
int32_t pars_gpu_flow_map_generate(pars_gpu_context* context, int32_t field, int32_t iterations, float resolution_scale,
                                   int32_t integrator, int32_t stage_mode, float step_size, int32_t* flow_map, int64_t* steps);
/* FTLE of a flow-map field: central-difference gradient (one-sided at the
 * borders), Cauchy-Green tensor C (FP32), then log(sqrt(lambda_max)) / |time|
 * with lambda_max from cyclic Jacobi rotations (mode REGULAR), or the
 * fractional anisotropy of C's eigenvalues (mode FRACTIONAL_ANISOTROPY,
 * ftle_map_generator.cpp:51-54).  Writes
 * the FP32 field to HOST `ftle` (X*Y*Z floats) unless it is NULL, in which case
 * the result stays on the device (pars_gpu_ftle_device_pointer). */
int32_t pars_gpu_ftle_generate    (pars_gpu_context* context, int32_t flow_map, float time, int32_t mode, float* ftle);
int32_t pars_gpu_ftle_device_pointer(pars_gpu_context* context, const float** device_ftle, int64_t* count);

/* ---- unsteady fields and batched advection ------------------------------------------
 * No counterpart in the reference (its fields are steady and its integrator
 * ignores time, particle_tracer.cpp:315-318).  An unsteady field holds
 * `slices` time slices of one grid, [slices][shape0][shape1][shape2][3] FP32;
 * slice k is the velocity at time t0 + k * slice_dt, linear in time between
 * slices and constant beyond the first and last slice. */
int32_t pars_gpu_unsteady_field_upload       (pars_gpu_context* context, const float* xyz, const int32_t shape[3], int32_t slices,
                                              const float offset[3], const float size[3], const float spacing[3],
                                              double t0, double slice_dt, int32_t* field);
int32_t pars_gpu_unsteady_field_upload_device(pars_gpu_context* context, const float* device_xyz, const int32_t shape[3],
                                              int32_t slices, const float offset[3], const float size[3],
                                              const float spacing[3], double t0, double slice_dt, int32_t* field);

/* One job of a batched advection: seeds on a (steady or unsteady) field,
 * advected with the flow-map rules of particle_advector
 * (particle_advector.cpp:74-139: stop on leaving the grid, on a zero velocity,
 * or after max_steps steps).  Pathlines on unsteady fields use classical RK4
 * in space-time with the time of step n = time_begin + n * step_size (about
 * 44 bits).  PARS_STAGES_FROZEN jobs run the reference's scheme bit for bit
 * (any of the eight integrators) on steady fields. */
typedef struct pars_gpu_batch_job
{
  int32_t      field;               /* field handle (steady or unsteady) */
  int32_t      integrator;          /* re-sampled stages: PARS_EULER or PARS_RUNGE_KUTTA_4; frozen: any */
  int32_t      stage_mode;          /* PARS_STAGES_RESAMPLED, or PARS_STAGES_FROZEN (steady fields) */
  int32_t      max_steps;
  float        step_size;
  int32_t      padding0;
  double       time_begin;          /* unsteady fields: start time */
  const float* seeds;               /* DEVICE float4 positions, or NULL for the lattice below */
  int64_t      seed_count;          /* seeds != NULL: number of seeds */
  float        lattice_offset[3];   /* seeds == NULL: offset + stride * index, C order (seed_generator.cpp:14-19) */
  float        lattice_stride[3];
  int32_t      lattice_count[3];
  int32_t      padding1;
  float*       end_positions;       /* DEVICE float4 per seed (last position; see below), may be NULL */
  int32_t*     end_steps;           /* DEVICE int32 per seed (steps taken), may be NULL */
  int64_t      steps;               /* out: particle-steps of this job */
} pars_gpu_batch_job;

/* End positions and flow maps of re-sampled stages are the correctly rounded
 * FP32 coordinates (x, y, z) and, in w, each coordinate's rounding residual as
 * a signed 10-bit code q (bits 0-9: x, 10-19: y, 20-29: z; bits 30-31 zero):
 * coordinate = x + q / 1022 * ulp(x), about 34 bits in all (the FTLE stage
 * differentiates flow maps with it).  Frozen-scheme results store w = 0. */
/* Advects every job in one persistent launch that drains a device queue of
 * seed chunks.  variant selects the launch shape (threads per CTA, register
 * budget) among pars_gpu_batch_variants(); -1 = autotuned: the first call of
 * each job class (steady / unsteady / frozen) on a device times every variant on
 * a probe of the batch and keeps the fastest for every context of that device in
 * the process.  Each class (re-sampled
 * steady, re-sampled unsteady, frozen) runs in its own launch. */
int32_t pars_gpu_batch_advect  (pars_gpu_context* context, pars_gpu_batch_job* jobs, int32_t count, int32_t variant);
int32_t pars_gpu_batch_variants(pars_gpu_context* context, int32_t* count);
/* The tuned variant of a job class (0 re-sampled steady, 1 re-sampled
 * unsteady, 2 frozen), -1 if not tuned yet. */
int32_t pars_gpu_batch_tuned   (pars_gpu_context* context, int32_t job_class, int32_t* variant, int32_t* threads);

/* ---- continuous batched advection --------------------------------------------------
 * The batched engine above with a job table that grows while it runs: jobs are
 * submitted at any time and join at the next horizon launch.  Each
 * pars_gpu_engine_advance runs one launch per job class with work, in which
 * every warp takes at most `iterations` steps and then parks its particles and
 * the rest of its seed pool in device memory; the next launch resumes them
 * before it starts the jobs submitted meanwhile.  A job's results (end
 * positions, step counts) are the same bits as pars_gpu_batch_advect's,
 * however its work is split into launches.  A job's field and output buffers
 * must stay valid until it is reported done.  Replaces, for a server, the
 * reference's one-request-at-a-time loop around particle_advector
 * (pars/source/service.cpp:41-68, pa/source/stages/particle_advector.cpp:74-139):
 * requests that arrive while others run share the device from the next
 * horizon on. */
typedef struct pars_gpu_engine_done
{
  int64_t ticket;
  int64_t steps;     /* particle-steps of the job */
} pars_gpu_engine_done;

/* Appends a job (same rules as pars_gpu_batch_advect; `steps` is ignored) and
 * returns its ticket.  The first job of a class tunes the class's launch shape
 * if the context has not tuned it yet. */
int32_t pars_gpu_engine_submit (pars_gpu_context* context, const pars_gpu_batch_job* job, int64_t* ticket);
/* One horizon launch per job class with work (iterations >= 1 steps per warp;
 * 0: the engine chooses the steps per launch for launches of about 2 ms from
 * the class's last launch, 256 for its first), then returns up to `capacity`
 * completed jobs (the rest on later calls) and, in *open, the jobs submitted
 * and not yet returned. */
int32_t pars_gpu_engine_advance(pars_gpu_context* context, int32_t iterations, pars_gpu_engine_done* done, int32_t capacity,
                                int32_t* done_count, int64_t* open);

/* ---- request service (pars_service, pars/source/service.cpp:20-69) ----------------
 * Requests are the reference's binary proto3 `settings` messages
 * (pars/proto/settings.proto).  `mode` is read as the reference reads it:
 * containing "ftle" selects the FTLE pipeline (pipeline::execute_ftle),
 * anything else streamlines (pipeline::execute: trace, prune, index, colour);
 * "fractional_anisotropy" selects the FA measure.  Integration uses
 * re-sampled RK4 stages; a mode containing "reference" traces streamlines
 * with the reference's frozen-velocity scheme instead.  `dataset_filepath`
 * names a dataset registered with pars_gpu_service_add_dataset.
 *
 * The service queues requests as they arrive.  `lanes` worker threads, each
 * with its own CUDA stream, take batches of queued requests of one kind that
 * fit into the device-memory budget (requests arriving while others run are
 * admitted as memory frees up).  A streamline batch runs as one tracing round
 * loop; FTLE requests run on the lane's continuous engine, which admits FTLE
 * requests that arrive while it runs at its next horizon launch and hands out
 * each request as soon as its own flow map completes
 * (pars_gpu_service_set_horizon).  A request's
 * results stay in device memory until the client copies them out
 * (pars_gpu_service_result_batch / _result_ftle, into any host buffers; pinned
 * ones copy fastest) and releases the request; held results count against
 * the budget.  When no queued request fits and no batch is running, held
 * results move to host memory, so a client that collects results in any order
 * cannot stall the queue.  Between batches the lanes keep up to budget / 4 of
 * scratch in total and the result pool up to budget / 4 of freed results, so
 * steady batches do not allocate: the service uses up to 1.5 x the budget of
 * device memory, plus the datasets. */
typedef struct pars_gpu_service pars_gpu_service;

/* The scalar fields of a decoded `settings` message (strings truncated). */
typedef struct pars_gpu_settings_summary
{
  char    mode[64];
  char    dataset_filepath[256];
  char    particle_tracing_integrator[64];
  char    color_generation_mode[64];
  int32_t seed_generation_stride[3];
  int32_t seed_generation_iterations;
  float   particle_tracing_step_size;
  int32_t particle_tracing_load_balance;
  float   color_generation_free_parameter;
  float   raytracing_camera_position[3];
  int32_t raytracing_image_size[2];
  float   raytracing_streamline_radius;
  int32_t raytracing_iterations;
} pars_gpu_settings_summary;

typedef struct pars_gpu_request_info
{
  int32_t state;          /* 0 queued, 1 running, 2 done */
  int32_t status;         /* PARS_OK or the failure */
  int32_t kind;           /* 0 streamlines, 1 FTLE */
  int32_t ftle_shape[3];
  int64_t batches;        /* streamlines: integral_curves batches */
  int64_t steps;          /* particle-steps taken */
  double  queue_ms;       /* submit -> start */
  double  run_ms;         /* start -> finish */
  double  latency_ms;     /* submit -> finish */
  int32_t image_size[2];  /* width, height of the request's image (0, 0 without one) */
} pars_gpu_request_info;

/* The binary `settings` message of its JSON form (the benchmark's settings
 * files, pars/source/service.cpp:72-77; the proto3 JSON mapping: field names
 * or lowerCamelCase names, numbers or numeric strings, unknown keys rejected).
 * *message_length receives the size; message (when not NULL, capacity large
 * enough) the bytes.  Host-only. */
int32_t pars_gpu_settings_from_json  (const char* json, int64_t length, uint8_t* message, int64_t capacity,
                                      int64_t* message_length);
/* Decodes a `settings` message (host-only; no device needed). */
int32_t pars_gpu_settings_decode     (const uint8_t* message, int64_t length, pars_gpu_settings_summary* settings);
int32_t pars_gpu_service_create      (pars_gpu_service** service, int32_t device, int64_t budget_bytes, int32_t lanes,
                                      int32_t max_batch);
int32_t pars_gpu_service_destroy     (pars_gpu_service* service);
/* FTLE requests run through the lane's continuous batched engine
 * (pars_gpu_engine_advance) with `iterations` steps per warp per launch
 * (default -1: chosen by the engine for launches of about 2 ms): between
 * launches finished requests are handed out and FTLE requests that arrived
 * meanwhile join the running launch sequence.  0 runs each FTLE batch to
 * completion in one launch instead.  Results are the same bits either way. */
int32_t pars_gpu_service_set_horizon (pars_gpu_service* service, int32_t iterations);
/* Registers a dataset (HOST xyz [X][Y][Z][3], as pars_gpu_field_upload) under `name`. */
int32_t pars_gpu_service_add_dataset (pars_gpu_service* service, const char* name, const float* xyz, const int32_t shape[3],
                                      const float offset[3], const float size[3], const float spacing[3]);
/* Same, from DEVICE xyz. */
int32_t pars_gpu_service_add_dataset_device(pars_gpu_service* service, const char* name, const float* device_xyz,
                                            const int32_t shape[3], const float offset[3], const float size[3],
                                            const float spacing[3]);
/* Registers a scalar volume (HOST values [X][Y][Z] FP32) under `name`, the
 * `volume_type` of requests whose mode contains "volume" (data_io.cpp:41-49). */
int32_t pars_gpu_service_add_volume  (pars_gpu_service* service, const char* name, const float* values, const int32_t shape[3],
                                      const float offset[3], const float spacing[3]);
int32_t pars_gpu_service_add_volume_device(pars_gpu_service* service, const char* name, const float* device_values,
                                           const int32_t shape[3], const float offset[3], const float spacing[3]);
/* Streamline requests whose settings carry raytracing_image_size (both > 0,
 * mode without "export") are also ray traced as pipeline.cpp:264-337 does:
 * camera position / forward / up (3 values each), radius (0 -> 1), iterations,
 * the volume named volume_type when the mode contains "volume" (a mode with
 * "volume" but not "streamlines" renders the volume alone). */
int32_t pars_gpu_service_submit      (pars_gpu_service* service, const uint8_t* message, int64_t length, int64_t* ticket);
/* Waits up to timeout_ms (negative: no limit, 0: poll) and reports the state;
 * returns the request's failure status once it has failed. */
int32_t pars_gpu_service_wait        (pars_gpu_service* service, int64_t ticket, int32_t timeout_ms, int32_t* state);
int32_t pars_gpu_service_result_info (pars_gpu_service* service, int64_t ticket, pars_gpu_request_info* info);
/* Streamline results, per batch: counts, then HOST copies (any pointer may be NULL). */
int32_t pars_gpu_service_result_batch(pars_gpu_service* service, int64_t ticket, int64_t batch, int64_t* vertices,
                                      int64_t* indices, float* vertex_data, float* color_data, int32_t* index_data);
/* FTLE results: ftle_shape[0]*ftle_shape[1]*ftle_shape[2] floats to HOST `values`. */
int32_t pars_gpu_service_result_ftle (pars_gpu_service* service, int64_t ticket, float* values);
/* The request's image (the reply of ray_tracer::serialize): size = (width,
 * height), (0, 0) without one; rgba (when not NULL) receives width*height*4
 * bytes, sRGB RGBA8, rows from the top.  pars_gpu_image_encode makes the
 * `image` message of it. */
int32_t pars_gpu_service_result_image(pars_gpu_service* service, int64_t ticket, uint8_t* rgba, int32_t size[2]);
/* Forgets a request (cancels it if it is still queued). */
int32_t pars_gpu_service_release     (pars_gpu_service* service, int64_t ticket);
/* Instrumentation (no counterpart in the reference's service; the reference
 * times its stages with its own benchmark recorder).  Enabling clears the
 * totals; from the next batch on, every lane times its kernels with CUDA
 * events and each batch phase by wall clock (the lane's stream is drained at
 * each phase end, so profiling costs some overlap).  Names: kernel names as
 * pars_gpu_profile_get reports them; phases "streamlines.seed",
 * "streamlines.trace", "streamlines.index_color", "streamlines.results",
 * "ftle.setup", "ftle.advect", "ftle.field", "lane.trim" (returning a lane's
 * scratch beyond what it keeps between batches) (milliseconds, count = batches);
 * "batches.streamlines" / "batches.ftle" (count = batches, milliseconds =
 * the number of requests they held). */
int32_t pars_gpu_service_profile_enable(pars_gpu_service* service, int32_t enable);
int32_t pars_gpu_service_profile_get   (pars_gpu_service* service, const char* name, double* milliseconds, int64_t* count);

/* ---- the service's transport (pars_service's ZeroMQ PAIR socket,
 * pars/source/service.cpp:20-69) ------------------------------------------------
 * ZMTP 3.0 (ZeroMQ RFC 23) over TCP with the NULL mechanism, as a PAIR socket,
 * without libzmq, so the reference's clients (a ZeroMQ PAIR socket that
 * connects and sends `settings` messages) talk to the service unchanged.
 * pars_gpu_transport_listen binds a TCP listener on an IPv4 address and port
 * (0: any free port, returned in *bound_port) and returns it in *listener.
 * pars_gpu_service_serve accepts one peer on it, answers each message with
 * the request's `image` message (pars_gpu_image_encode; width and height 0
 * when the request made no image or failed), and returns once the peer
 * closes or max_requests messages (<= 0: no limit) were answered; *served
 * receives the count.  It blocks the calling thread; call it again for the
 * next peer.  Host-only; the service does the GPU work. */
int32_t pars_gpu_transport_listen(const char* address, int32_t port, int32_t* bound_port, int64_t* listener);
int32_t pars_gpu_transport_close (int64_t listener);
int32_t pars_gpu_service_serve   (pars_gpu_service* service, int64_t listener, int64_t max_requests, int64_t* served);

/* ---- allocation-free FTLE --------------------------------------------------------
 * No counterpart in the reference.  For callers that may not allocate device
 * memory: plugins running inside a host application that owns the GPU's
 * memory budget (an in-situ simulation, a renderer), and paths where the
 * implicit synchronisation of cudaMalloc / cudaFree is not acceptable.  It
 * needs no context and calls no cudaMalloc, cudaFree or allocating library
 * routine: the flow map and the float4 copy of the field live in one static
 * device array of this library (8 MiB, held on every GPU that loads the
 * library until the process exits).
 *
 * Computes what pars_gpu_field_upload_device + pars_gpu_flow_map_generate
 * (resolution scale 1) + pars_gpu_ftle_generate compute (bit for bit with
 * frozen stages; to rounding with re-sampled RK4 / Euler, which the context
 * path runs through its batched engine), on the CURRENT CUDA
 * device and `stream` (a cudaStream_t, NULL = default stream): device_xyz is
 * the field in DEVICE memory ([shape0][shape1][shape2][3] FP32), device_ftle
 * receives shape0*shape1*shape2 FP32 values in DEVICE memory, and
 * device_steps (DEVICE int64, may be NULL) the particle-steps taken.
 * Limit: shape0*shape1*shape2 <= 262144 (64^3); larger fields (or any
 * shape entry above that) return PARS_ERR_BUDGET before any CUDA call.
 * int(size / spacing) must lie between shape and shape + 1 per axis (one
 * seed per vertex), else PARS_ERR_INVALID_ARGUMENT.
 * The first call on a device looks up the array's device address (once per
 * device, with that device current); make that first call before any stream
 * capture.  The address is cached per device ordinal for the process's
 * lifetime: only the device's primary context (the CUDA runtime's) is
 * supported, and after cudaDeviceReset the process must restart before it
 * calls this again.  All calls share the one array: calls that overlap on the GPU
 * (different streams or threads without ordering between them) race and
 * corrupt each other's results; order them on one stream. */
int32_t pars_gpu_ftle_no_alloc(const float* device_xyz, const int32_t shape[3], const float offset[3], const float size[3],
                               const float spacing[3], int32_t iterations, int32_t integrator, int32_t stage_mode,
                               float step_size, float time, int32_t mode, float* device_ftle, int64_t* device_steps,
                               void* stream);

/* ---- field files (replaces pa::data_io, pa/source/stages/data_io.cpp) -------------------
 * HDF5 is not part of this library; datasets live in "pars raw" files: a
 * 64-byte header (magic "PARSRAW1", uint32 components (3: vector field, 1:
 * scalar field), uint32 0, int64 shape[3], float spacing[3], zero padding)
 * and FP32 data [shape0][shape1][shape2][components], little endian.  Host-only
 * unless a context is passed. */
/* data_io::load_dimensions (data_io.cpp:36-40): components, shape and raw spacing. */
int32_t pars_gpu_raw_info (const char* path, int32_t* components, int64_t shape[3], float spacing[3]);
/* Writes a whole dataset (e.g. converted from HDF5). */
int32_t pars_gpu_raw_write(const char* path, int32_t components, const int64_t shape[3], const float spacing[3],
                           const float* data);
/* data_io::load_local_vector_field (data_io.cpp:50-58, 90-114): the ghosted
 * block of rank `rank` of `ranks` (pars_gpu_partition) as a resident field:
 * spacing divided by its maximum, offset = voxel offset x spacing, size = block
 * size x spacing.  *partition (may be NULL) receives the block's geometry. */
int32_t pars_gpu_field_load(pars_gpu_context* context, const char* path, int32_t ranks, int32_t rank, int32_t* field,
                            pars_partition_info* partition);
/* data_io::load_scalar_field (data_io.cpp:41-49, 76-89) into HOST values
 * [shape0][shape1][shape2] (NULL: geometry only). */
int32_t pars_gpu_scalar_load(const char* path, int32_t ranks, int32_t rank, float* values, int32_t shape[3], float offset[3],
                             float spacing[3], float size[3]);
/* data_io::save_ftle_field (data_io.cpp:117-140): writes a block of FTLE values
 * ([shape0][shape1][shape2] at voxel `offset`) into the scalar file of the
 * whole `domain`, creating it (zero-filled, with `spacing`) when missing. */
int32_t pars_gpu_ftle_save(const char* path, const int32_t domain[3], const int32_t offset[3], const int32_t shape[3],
                           const float* values, const float spacing[3]);

/* data_io::save_integral_curves (data_io.cpp:142-196): the curves as VTK XML
 * PolyData (.vtp, raw appended data): non-termination vertices as points with
 * colour bytes (x 255, rounded, clamped; "Colors"), one polyline per run ended
 * by a termination vertex.  _export_vtk takes host batches (colors or an
 * entry may be NULL), _curves_export_vtk the context's device curves. */
int32_t pars_gpu_export_vtk(const char* path, int64_t batches, const int64_t* vertex_counts, const float* const* vertices,
                            const float* const* colors);
int32_t pars_gpu_curves_export_vtk(pars_gpu_context* context, const char* path);

/* ---- ray tracer (replaces pars::ray_tracer, pars/include/pars/stages/ray_tracer.hpp:27-34) ----
 * One ray tracer per context.  Scene: one capsule (cylinder plus end spheres)
 * of the given radius per line index, coloured with vertex colour[index];
 * optionally a scalar volume with the reference's transfer function (grey
 * ramp, opacity 0.0001 -> 0.0255 over values 0 -> 1).  Camera: perspective,
 * fovy 68 degrees.  Lights: ambient 1 and the two distant lights of
 * ray_tracer.cpp:68-91.  Frames accumulate (one sample per pixel each, jittered
 * after the first) until the scene, camera or image size changes.  The
 * shading is this library's definition of that configuration (OSPRay is not
 * involved); the image is sRGB-encoded RGBA8, rows from the top. */
/* ray_tracer::set_volume (ray_tracer.cpp:130-163): values [X][Y][Z] FP32 (z fastest),
 * host memory (_device: device memory; both are copied). */
int32_t pars_gpu_ray_tracer_set_volume       (pars_gpu_context* context, const float* values, const int32_t shape[3],
                                              const float offset[3], const float spacing[3]);
int32_t pars_gpu_ray_tracer_set_volume_device(pars_gpu_context* context, const float* device_values, const int32_t shape[3],
                                              const float offset[3], const float spacing[3]);
int32_t pars_gpu_ray_tracer_clear_volume     (pars_gpu_context* context);
/* ray_tracer::set_integral_curves (ray_tracer.cpp:164-211) on the context's
 * device-resident curves (after pars_gpu_curves_index, and _color for
 * colours; uncoloured curves render white).  The curves are used in place:
 * tracing, indexing or colouring again makes _trace fail with PARS_ERR_STATE
 * until this is called again.  radius > 0 (pipeline.cpp:306 passes 1 for 0). */
int32_t pars_gpu_ray_tracer_set_integral_curves(pars_gpu_context* context, float radius);
/* The same for host batches (pa::integral_curves vectors): per batch its
 * vertex count, vertices (float4), colours (float4; colors or an entry NULL:
 * white), index count and indices; batches without indices are skipped. */
int32_t pars_gpu_ray_tracer_set_integral_curves_host(pars_gpu_context* context, int64_t batches, const int64_t* vertex_counts,
                                                     const float* const* vertices, const float* const* colors,
                                                     const int64_t* index_counts, const int32_t* const* indices, float radius);
/* ray_tracer::set_camera (ray_tracer.cpp:213-220) and set_image_size (:221-229). */
int32_t pars_gpu_ray_tracer_set_camera    (pars_gpu_context* context, const float position[3], const float forward[3],
                                           const float up[3]);
int32_t pars_gpu_ray_tracer_set_image_size(pars_gpu_context* context, int32_t width, int32_t height);
/* ray_tracer::trace (ray_tracer.cpp:231-235): adds `iterations` frames. */
int32_t pars_gpu_ray_tracer_trace         (pars_gpu_context* context, int32_t iterations);
/* ray_tracer::serialize (ray_tracer.cpp:236-253): the image's size and, when
 * rgba is not NULL, its width*height*4 bytes (sRGB RGBA8) of the average of
 * the frames so far (background before the first frame). */
int32_t pars_gpu_ray_tracer_serialize     (pars_gpu_context* context, uint8_t* rgba, int32_t size[2]);
/* Frames accumulated since the last change. */
int32_t pars_gpu_ray_tracer_frames        (pars_gpu_context* context, int64_t* frames);
/* Encodes the `image` message (pars/proto/image.proto): *length receives the
 * encoded size; out (when not NULL, with capacity >= that size) the bytes. */
int32_t pars_gpu_image_encode(const int32_t size[2], const uint8_t* data, int64_t data_bytes, uint8_t* out, int64_t capacity,
                              int64_t* length);

/* ---- instrumentation ---------------------------------------------------------- */
/* When enabled, each kernel launch is bracketed by CUDA events on the launch
 * stream and its time is accumulated per kernel name. */
int32_t pars_gpu_profile_enable(pars_gpu_context* context, int32_t enable);
int32_t pars_gpu_profile_reset (pars_gpu_context* context);
/* Accumulated time and launches of the kernel called `name` (0 if never run). */
int32_t pars_gpu_profile_get   (pars_gpu_context* context, const char* name, double* milliseconds, int64_t* launches);
/* Kernel launches issued by this library on the context since creation. */
int32_t pars_gpu_launch_count  (pars_gpu_context* context, int64_t* launches);
/* Gather-bandwidth calibration (no counterpart in the reference; the measured
 * ceilings for the advection kernels' roofline).  Times 16-byte non-coherent
 * loads, the instruction the kernels use for cell corners, into a zeroed
 * device buffer of buffer_bytes (rounded down to a power of two, 4 KiB to
 * 64 GiB) on the context's stream.  pattern 0: each warp request reads 512
 * contiguous bytes at a random aligned offset; 1: each lane 16 bytes at its
 * own random offset; 2: each lane the eight corners of a random cell of a
 * cube float4 field.  *bytes_per_second receives the bytes delivered to
 * registers per second.  32 KiB stays in L1, 64 MiB in L2. */
int32_t pars_gpu_gather_peak   (pars_gpu_context* context, int64_t buffer_bytes, int32_t pattern, double* bytes_per_second);

#ifdef __cplusplus
}
#endif

#endif /* PARS_GPU_H */
