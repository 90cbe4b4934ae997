/* hbtu.h -- C ABI of the GB300 (sm_103a) subhalo-unbinding library.
 *
 * Drop-in replacement for HBT+'s unbinding step:
 *   void Subhalo_t::Unbind(const Snapshot_t &epoch)
 *     src/subhalo.h:111, src/subhalo_unbind.cpp:263-431
 * and for the per-subhalo loops of its caller
 *   void SubhaloSnapshot_t::RefineParticles()   src/subhalo_unbind.cpp:460-516
 * (gather all subhaloes of one nesting level into one batch call).
 *
 * Plain C: no exceptions cross it, every call returns an hbtu_status, buffers
 * are owned by the caller.  One handle = one CUDA stream and one device
 * workspace; calls on different handles may run concurrently from different
 * host threads; calls on one handle must not overlap.
 */
#ifndef HBTU_H
#define HBTU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum hbtu_status {
  HBTU_OK = 0,
  HBTU_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size or parameter */
  HBTU_ERR_CUDA = 2,             /* a CUDA runtime call failed (see hbtu_last_error) */
  HBTU_ERR_OUT_OF_MEMORY = 3,    /* device workspace could not be allocated */
  HBTU_ERR_NOT_CONVERGED = 4,    /* a subhalo hit max_passes (see hbtu_result.status) */
  HBTU_ERR_NO_DEVICE = 5,        /* no CUDA device of compute capability 10.3 */
  HBTU_ERR_TOO_LARGE = 6         /* more than HBTU_MAX_PARTICLES particles in one call */
} hbtu_status;

#define HBTU_MAX_PARTICLES ((int64_t)1 << 30)

typedef enum hbtu_precision {
  HBTU_PRECISION_FP32 = 0, /* walk in FP32 on coordinates relative to the subhalo,
                              FP64 sums for frames and convergence (default) */
  HBTU_PRECISION_FP64 = 1  /* walk in FP64 with the reference's operation order */
} hbtu_precision;

typedef enum hbtu_location { HBTU_HOST = 0, HBTU_DEVICE = 1 } hbtu_location;

/* Unbinding parameters: the subset of HBT+'s Parameter_t read by Unbind
 * (src/config_parser.h:22-123), the snapshot's cosmology and G.  Values are
 * rounded to float (HBTReal) exactly as the reference stores them. */
typedef struct hbtu_params {
  double softening;            /* SofteningHalo (compulsory) */
  double open_angle;           /* TreeNodeOpenAngle, default 0.45 */
  double bound_mass_precision; /* BoundMassPrecision, default 0.995 */
  int64_t min_num_part;        /* MinNumPartOfSub, default 20 */
  int64_t max_sample_size;     /* MaxSampleSizeOfPotentialEstimate, default 1000; 0 = exact */
  int32_t refine_mostbound;    /* RefineMostboundParticle, default 1 */
  int32_t periodic;            /* PeriodicBoundaryOn, default 1 */
  double box_size;             /* BoxSize */
  double G;                    /* PhysicalConst::G = 43.0071*(MassInMsunh/1e10)/VelInKmS^2/LengthInMpch */
  double hubble;               /* Cosmology.Hz of the snapshot (internal units) */
  double scale_factor;         /* Cosmology.ScaleFactor of the snapshot */
  int32_t precision;           /* hbtu_precision */
  int32_t max_passes;          /* cap on loop passes per subhalo (0 = 10000) */
  int32_t device;              /* CUDA device ordinal */
  int32_t reserved;
} hbtu_params;

/* Per-subhalo state read by Unbind besides its particles. */
typedef struct hbtu_state {
  float ref_pos[3];       /* ComovingAveragePosition: initial frame */
  float ref_vel[3];       /* PhysicalAverageVelocity: initial frame */
  float mostbound_pos[3]; /* ComovingMostBoundPosition (restored on disruption) */
  float mostbound_vel[3]; /* PhysicalMostBoundVelocity (restored on disruption) */
  int64_t mostbound_id;   /* Id of the previous most-bound particle (Particles[0]
                             before the sampling shuffle) */
} hbtu_state;

/* Per-subhalo outputs: the Subhalo_t members Unbind writes (src/subhalo.h:29-91). */
typedef struct hbtu_result {
  int64_t nbound;           /* Nbound */
  float mbound;             /* Mbound */
  float ref_pos[3];         /* ComovingAveragePosition */
  float ref_vel[3];         /* PhysicalAverageVelocity */
  float mostbound_pos[3];   /* ComovingMostBoundPosition */
  float mostbound_vel[3];   /* PhysicalMostBoundVelocity */
  float specific_potential; /* SpecificSelfPotentialEnergy */
  float specific_kinetic;   /* SpecificSelfKineticEnergy */
  float specific_angmom[3]; /* SpecificAngularMomentum */
  int64_t nbound_type[6];   /* NboundType */
  float mbound_type[6];     /* MboundType */
  int32_t iterations;       /* passes of the unbinding loop */
  int32_t disrupted;        /* the disruption branch ran: set SnapshotIndexOfDeath if alive */
  int32_t converged;        /* converged: clear death (if dead) and sink (if trapped) */
  int32_t too_few;          /* n < MinNumPartOfSub: set SnapshotIndexOfDeath if alive */
  int64_t evaluations;      /* target potentials evaluated */
  int64_t interactions;     /* tree-walk contributions summed */
  int32_t status;           /* 0 ok, HBTU_ERR_NOT_CONVERGED if max_passes was hit */
  int32_t reserved;
} hbtu_result;

/* Particle arrays of one call (n particles, or the concatenation of a batch).
 * pos and vel hold 3 floats per particle (HBTxyz), like Particle_t. */
typedef struct hbtu_particles {
  const int64_t *id;   /* Particle_t::Id */
  const float *pos;    /* Particle_t::ComovingPosition, 3n */
  const float *vel;    /* Particle_t::PhysicalVelocity, 3n */
  const float *mass;   /* Particle_t::Mass */
  const int32_t *type; /* Particle_t::Type (0..5), may be NULL (all TypeDM) */
  int32_t location;    /* hbtu_location of these arrays AND of the output arrays */
  int32_t reserved;
} hbtu_particles;

typedef struct hbtu_handle hbtu_handle;

/* Create a handle on params->device, with its own stream and workspace.
 * Replaces the configuration read of Parameter_t::ParseConfigFile
 * (src/config_parser.cpp:74-109) for the unbinding subset. */
hbtu_status hbtu_create(const hbtu_params *params, hbtu_handle **out);
hbtu_status hbtu_destroy(hbtu_handle *h);

/* Enqueue the handle's work on a caller-owned cudaStream_t from now on.
 * NULL is CUDA's legacy default stream (what a framework's "current stream"
 * is by default), so work there is ordered with the caller's.  A new handle
 * uses a stream of its own.  The library's kernels are launched with
 * programmatic stream serialisation: each is scheduled while the kernel
 * before it still runs, and waits (griddepcontrol.wait) for that kernel to
 * complete before it touches memory, so stream order is kept, also after the
 * caller's own kernels.  HBTU_LAUNCH_OVERLAP=0 in the environment launches
 * them the plain way. */
hbtu_status hbtu_set_stream(hbtu_handle *h, void *cuda_stream);

/* Unbind one subhalo: Subhalo_t::Unbind (src/subhalo_unbind.cpp:263-431).
 *   p, n:       its particles; position 0 = the previous most-bound particle
 *               (when sampling applies the caller has applied the reference's
 *               random_shuffle first, src/subhalo_unbind.cpp:302)
 *   st:         frame and most-bound record on entry (host memory)
 *   order_out:  n int64; output position i holds input particle order_out[i]
 *               (the permuted Particles vector)
 *   energy_out: n float; binding energy at output position i; the first
 *               nbound are Subhalo_t::Energies (SAVE_BINDING_ENERGY)
 *   res:        one hbtu_result (same location as the particle arrays) */
hbtu_status hbtu_unbind(hbtu_handle *h, const hbtu_particles *p, int64_t n,
                        const hbtu_state *st, int64_t *order_out, float *energy_out,
                        hbtu_result *res);

/* Unbind nsub independent subhaloes in one device-resident loop: the
 * per-subhalo Unbind calls of SubhaloSnapshot_t::RefineParticles
 * (src/subhalo_unbind.cpp:471-513) for one nesting level.
 *   offsets: nsub+1 int64 (host memory); subhalo s owns particles
 *            [offsets[s], offsets[s+1]) of p
 *   st:      nsub states (host memory)
 *   order_out / energy_out: per particle, positions local to each subhalo
 *   res:     nsub results (same location as the particle arrays) */
hbtu_status hbtu_unbind_batch(hbtu_handle *h, const hbtu_particles *p, int64_t nsub,
                              const int64_t *offsets, const hbtu_state *st, int64_t *order_out,
                              float *energy_out, hbtu_result *res);

/* One energy pass: a tree over all n particles and, for each,
 * GravityTree_t::BindingEnergy (src/gravity_tree.cpp:166-175) with the
 * self-term cancelled -- the first pass of the unbinding loop
 * (src/subhalo_unbind.cpp:333-354).  potential_out (may be NULL) receives
 * GravityTree_t::EvaluatePotential (src/gravity_tree.cpp:79-164). */
hbtu_status hbtu_binding_energies(hbtu_handle *h, const hbtu_particles *p, int64_t n,
                                  const float ref_pos[3], const float ref_vel[3],
                                  float *energy_out, double *potential_out);

/* Largest subhalo hbtu_unbind_noalloc accepts (its fixed scratch capacity). */
#define HBTU_NOALLOC_MAX_PARTICLES 16384

/* hbtu_unbind for callers that cannot allocate GPU memory (code running
 * inside another framework's memory pool, a process whose device memory is
 * reserved up front, a pipeline that forbids allocation after start-up).  No
 * counterpart in the reference: it is an addition of this library.
 *   - no handle: params as for hbtu_create; runs on the current device and on
 *     cuda_stream (NULL: the default stream);
 *   - p, order_out, energy_out and res must all be device memory
 *     (p->location == HBTU_DEVICE); st is host memory;
 *   - working memory is a fixed 8 MiB array inside the library, held by every
 *     GPU that loads it until exit; subhaloes of more than
 *     HBTU_NOALLOC_MAX_PARTICLES particles return HBTU_ERR_TOO_LARGE;
 *   - the first call on a device looks up the array's device address; make
 *     that call before any stream capture;
 *   - all calls share the array: calls that overlap on the GPU race, so
 *     serialise them;
 *   - it calls no cudaMalloc, cudaFree or other allocating routine.
 * Errors are reported by hbtu_last_error(NULL). */
hbtu_status hbtu_unbind_noalloc(const hbtu_params *params, const hbtu_particles *p, int64_t n,
                                const hbtu_state *st, int64_t *order_out, float *energy_out,
                                hbtu_result *res, void *cuda_stream);

/* Counters and device timings accumulated by a handle (tracing). */
typedef struct hbtu_stats {
  double total_ms;         /* device time of the unbinding calls, CUDA events on the handle's stream */
  double tree_ms;          /* with timing on: octree builds (keys, sort, cells, moments) */
  double walk_ms;          /* with timing on: the Barnes-Hut energy walks */
  double loop_ms;          /* with timing on: partition, averages, control, energy sorts */
  int64_t calls;           /* unbinding calls */
  int64_t passes;          /* loop passes (all subhaloes of a call advance together) */
  int64_t kernel_launches; /* CUDA kernels launched by the library */
  int64_t walk_launches;   /* of which tree walks */
  int64_t evaluations;     /* target potentials evaluated */
  int64_t interactions;    /* tree-walk contributions summed */
  double walk1_ms;         /* with timing on: the first pass's walk of each call */
  int64_t walk1_interactions; /* contributions summed by those first-pass walks */
  double small_ms;         /* with timing on: the per-subhalo loop (option "small_cutoff") */
  int64_t small_subhaloes; /* subhaloes whose last passes ran in it */
} hbtu_stats;

/* Turn per-phase device timing on (1) or off (0; the default).  With timing
 * off only total_ms and the counters are kept. */
hbtu_status hbtu_set_timing(hbtu_handle *h, int32_t on);
hbtu_status hbtu_get_stats(const hbtu_handle *h, hbtu_stats *out);
hbtu_status hbtu_reset_stats(hbtu_handle *h);

/* Tuning options of a handle (results do not depend on them):
 *   "small_cutoff"    (default 2048, at most 2048; 0: off) from the first
 *                     round of the loop at which every active subhalo's
 *                     energy list holds at most this many particles, one
 *                     persistent launch finishes them all, one thread block
 *                     per subhalo running its remaining passes (a work queue
 *                     in size order); before it, every active subhalo
 *                     advances one pass per round of batch kernels.  With
 *                     walk_schedule 1 it is off.
 *   "small_blocks_per_sm" (default 1, 1..8) blocks per SM of that launch.
 *   "walk_schedule"   how the FP32 walk visits nodes: 0 (default) every
 *                     lane walks its own target; 1 a warp visits the smallest
 *                     node index any of its targets waits at (broadcast loads).
 *   "walk_leaf_runs"  1 (default) or 0: with walk_schedule 1, stream the
 *                     particles of a cell whose children are all particles.
 *   "walk_layout"     1 (default) or 0: with walk_schedule 0, passes whose
 *                     trees hold at least 2^16 particles in all walk a copy
 *                     of the node records with every cell's children in
 *                     consecutive slots (0: the preorder records). */
hbtu_status hbtu_set_option(hbtu_handle *h, const char *name, int64_t value);
hbtu_status hbtu_get_option(const hbtu_handle *h, const char *name, int64_t *value);

/* Adjoint of the binding energy: the gradient of each subhalo's total binding
 * energy over a fixed particle set (e.g. its bound particles after unbinding),
 *   E_tot = sum_i m_i |dv_i|^2 / 2 + 1/2 sum_i m_i phi_i,
 * dv_i = RelativeVelocity(x_i, v_i, ref_pos, ref_vel) (src/snapshot.h:100-111),
 * phi_i the tree potential of the unbinding walk (src/gravity_tree.cpp:79-164).
 * No counterpart in the reference.  With the frame at the set's centre of mass:
 *   dE/dv = m dv,  dE/dx = m (H a dv + grad phi),  dE/dm = |dv|^2 / 2 + phi,
 * grad phi from a walk with the reference's opening rule (recomputed, nothing
 * stored).  Batched like hbtu_unbind_batch: offsets (host), st[nsub] (host,
 * ref_pos/ref_vel used), energy_out[nsub] double; grad_pos[3N], grad_vel[3N],
 * grad_mass[N] float by input position, each may be NULL; arrays follow
 * p->location. */
hbtu_status hbtu_energy_gradient(hbtu_handle *h, const hbtu_particles *p, int64_t nsub,
                                 const int64_t *offsets, const hbtu_state *st, double *energy_out,
                                 float *grad_pos, float *grad_vel, float *grad_mass);

/* Validation utility (no counterpart in the reference): exact pairwise
 * potentials in FP64 of the particles targets[0..ntarget) (indices into p)
 * from all n particles of p, with the reference's spline softening and
 * periodic wrap, times G/a -- the quantity GravityTree_t::EvaluatePotential
 * approximates (src/gravity_tree.cpp:79-164).  targets and potential_out are
 * host memory; p follows p->location. */
hbtu_status hbtu_direct_potential(hbtu_handle *h, const hbtu_particles *p, int64_t n,
                                  const int64_t *targets, int64_t ntarget, double *potential_out);

/* Post-unbinding properties of a subhalo: the members of Subhalo_t written
 * by CalculateProfileProperties (src/subhalo.cpp:242-335) and CalculateShape
 * (src/subhalo.cpp:337-398). */
typedef struct hbtu_props {
  float rmax_comoving;              /* RmaxComoving */
  float vmax_physical;              /* VmaxPhysical */
  float last_max_vmax_physical;     /* LastMaxVmaxPhysical (updated) */
  int32_t snapshot_of_last_max_vmax; /* SnapshotIndexOfLastMaxVmax (updated) */
  float r2sigma_comoving;           /* R2SigmaComoving */
  float rhalf_comoving;             /* RHalfComoving */
  float r200crit_comoving;          /* BoundR200CritComoving */
  float m200crit;                   /* BoundM200Crit */
  float inertial_tensor[6];         /* InertialTensor {xx, xy, xz, yy, yz, zz} */
  float inertial_tensor_weighted[6]; /* InertialTensorWeighted */
} hbtu_props;

/* CalculateProfileProperties + CalculateShape of every subhalo of a batch
 * that hbtu_unbind_batch (or hbtu_unbind, nsub = 1) has just unbound, on the
 * first nbound particles of each subhalo's output order.
 *   p, nsub, offsets: the particles and offsets given to the unbinding
 *     (offsets in host memory; pos and mass are read);
 *   order, res: its order_out and res, in the memory p->location names;
 *   last_max_vmax, last_snap: nsub values of LastMaxVmaxPhysical and
 *     SnapshotIndexOfLastMaxVmax before the call (host memory; NULL: 0 and -1);
 *   snapshot_index: the epoch's snapshot index (Snapshot_t::GetSnapshotIndex);
 *   out: nsub records (host memory).
 * G, Hz and the scale factor come from the handle's parameters; the
 * overdensity is 200 times critical (Snapshot_t::HaloVirialFactors,
 * src/snapshot.cpp:328-336).  A subhalo with nbound <= 1 gets zeros and its
 * last-maximum fields unchanged, as in the reference.  Distance ties keep the
 * unbinding order; the inertia tensors may differ from the reference's
 * sequential sums by one unit in the last place (the order of the double
 * sum); every other field is exact. */
hbtu_status hbtu_subhalo_properties(hbtu_handle *h, const hbtu_particles *p, int64_t nsub,
                                    const int64_t *offsets, const int64_t *order,
                                    const hbtu_result *res, const float *last_max_vmax,
                                    const int32_t *last_snap, int32_t snapshot_index,
                                    hbtu_props *out);

/* Core of a subhalo as the merging step sees it (SubHelper_t,
 * src/subhalo_merge.cpp:14-26): mean position and velocity of its first
 * min(Nbound, 20) particles (NumPartCoreMax) and their dispersions. */
typedef struct hbtu_core {
  float pos[3];   /* ComovingPosition */
  float sigma_r;  /* ComovingSigmaR */
  float vel[3];   /* PhysicalVelocity */
  float sigma_v;  /* PhysicalSigmaV */
} hbtu_core;

/* FillCores + DetectTraps, the first half of SubhaloSnapshot_t::MergeSubhalos
 * (src/subhalo_merge.cpp:30-180, :187-199), for every subhalo at once.
 *   p: the particles of every subhalo's list, concatenated, bound first
 *      (list_off: nsub+1 offsets, host memory); pos, vel and mass are read;
 *   nbound[s]: Nbound; host[s]: HostTrackId as local index (-1: none; the
 *      other top-level subhaloes of a halo count as nested in its central,
 *      GlueHeadNests); mostbound_pos/vel[3*s]: ComovingMostBoundPosition,
 *      PhysicalMostBoundVelocity;
 *   sink[s]: SinkTrackId on entry (-1: not trapped; such a subhalo is skipped)
 *      and on return; a subhalo trapped now gets sink_snap[s] = snapshot_index
 *      (other entries are left as given); merged[s] = 1 marks a subhalo that
 *      swallows a subhalo with Nbound > 1 (Helpers[].IsMerged), else 0;
 *   cores (may be NULL): every subhalo's core.
 * All arrays but p's are host memory.  The merge itself (MergeTo: the union
 * of particle lists by Id) and the re-unbinding of merged subhaloes
 * (hbtu_unbind_batch) follow on the caller's side.  A host chain with a
 * cycle returns HBTU_ERR_INVALID_ARGUMENT. */
hbtu_status hbtu_merge_detect(hbtu_handle *h, const hbtu_particles *p, int64_t nsub,
                              const int64_t *list_off, const int64_t *nbound, const int64_t *host,
                              const float *mostbound_pos, const float *mostbound_vel,
                              int32_t snapshot_index, int64_t *sink, int32_t *sink_snap,
                              int32_t *merged, hbtu_core *cores);

/* Particle-ID -> index tables, the ID re-resolve of the unbinding step's
 * callers (IndexTable_t, src/hash.h:47-112; filled from a snapshot's IDs by
 * ParticleSnapshot_t, src/snapshot.h:191-224, and queried by GetIndex /
 * GetIndices, src/hash.tpp:47-55 / src/hash_remote.tpp:5-99).  A table lives
 * on the handle's device and uses its stream.
 *   flat = 0: MappedIndexTable_t (pairs sorted by key, binary search per
 *             query; a negative key is absent) -- here a hash table with the
 *             same answers, no sort;
 *   flat = 1: FlatIndexTable_t -- a dense array over [KeyMin, KeyMax] (key
 *             spans above 2^32 are refused: HBTU_ERR_TOO_LARGE).
 * Duplicate keys (undefined in the reference): the first pair in input order
 * wins in a mapped table, the last in a flat table. */
typedef struct hbtu_index_table hbtu_index_table;
hbtu_status hbtu_index_create(hbtu_handle *h, int32_t flat, hbtu_index_table **out);
hbtu_status hbtu_index_destroy(hbtu_index_table *t);
/* IndexTable_t::Fill(Keys, null_index) (src/hash.tpp:18-30, :59-95): the
 * pairs (keys[i], values[i]), i < n (KeyList_t::GetKey / ::GetIndex); both
 * arrays in host (location HBTU_HOST) or device memory. */
hbtu_status hbtu_index_fill(hbtu_index_table *t, const int64_t *keys, const int64_t *values,
                            int64_t n, int64_t null_index, int32_t location);
/* GetIndex for every query: out[j] = the value paired with keys[j], or the
 * null index (GetIndices, any query order); keys and out in host or device
 * memory as location says. */
hbtu_status hbtu_index_lookup(hbtu_index_table *t, const int64_t *keys, int64_t m, int64_t *out,
                              int32_t location);
/* GetKeyMinMax (src/hash.h:88-93, :102-107); max < min for an empty table. */
hbtu_status hbtu_index_key_range(const hbtu_index_table *t, int64_t *key_min, int64_t *key_max);

/* Message of the last failed call on this handle (or of the last failed
 * hbtu_create when h is NULL). */
const char *hbtu_last_error(const hbtu_handle *h);

/* Library version, as major*10000 + minor*100 + patch. */
int32_t hbtu_version(void);

#ifdef __cplusplus
}
#endif
#endif /* HBTU_H */
