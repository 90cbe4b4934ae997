/* hbt_oracle.h -- CPU oracle for the HBT+ subhalo-unbinding path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (Subhalo_t::Unbind, src/subhalo_unbind.cpp:263-431, with the octree
 * of src/oct_tree.tpp:16-144 and the potential walk of src/gravity_tree.cpp:18-175)
 * used as the checker for the GPU implementation and as the timed CPU baseline.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may call it; the
 * product path (hbtplus_gb300/) never links or executes anything from here.
 *
 * The same entry points are exported, with the prefix ref_ instead of hbto_,
 * by oracle/ref/ref_driver.cpp, which wraps the reference's own compiled
 * Subhalo_t::Unbind.  The oracle is pinned against that build (tests/).
 */
#ifndef HBT_ORACLE_H
#define HBT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Unbinding parameters, named after the reference's Parameter_t members
 * (src/config_parser.h:22-123).  Values are rounded to float (HBTReal) on
 * entry, exactly as the reference stores them. */
typedef struct hbto_params {
  double softening;            /* SofteningHalo */
  double open_angle;           /* TreeNodeOpenAngle */
  double bound_mass_precision; /* BoundMassPrecision */
  int64_t min_num_part;        /* MinNumPartOfSub */
  int64_t max_sample_size;     /* MaxSampleSizeOfPotentialEstimate (0 = exact) */
  int32_t refine_mostbound;    /* RefineMostboundParticle */
  int32_t periodic;            /* PeriodicBoundaryOn */
  double box_size;             /* BoxSize */
  double G;                    /* PhysicalConst::G */
  double hubble;               /* Cosmology.Hz of the snapshot */
  double scale_factor;         /* Cosmology.ScaleFactor of the snapshot */
} hbto_params;

/* Per-subhalo state on entry to Unbind: the Subhalo_t members it reads
 * besides Particles (src/subhalo_unbind.cpp:264, :298, :375-376). */
typedef struct hbto_state {
  float ref_pos[3];       /* ComovingAveragePosition (initial frame) */
  float ref_vel[3];       /* PhysicalAverageVelocity (initial frame) */
  float mostbound_pos[3]; /* ComovingMostBoundPosition (restored on disruption) */
  float mostbound_vel[3]; /* PhysicalMostBoundVelocity (restored on disruption) */
  int64_t mostbound_id;   /* Id of Particles[0] before any shuffle */
} hbto_state;

/* Per-subhalo outputs: the Subhalo_t members that Unbind writes
 * (src/subhalo.h:29-91), plus counters the reference does not keep. */
typedef struct hbto_result {
  int64_t nbound;                 /* Nbound */
  float mbound;                   /* Mbound */
  float ref_pos[3];               /* ComovingAveragePosition */
  float ref_vel[3];               /* PhysicalAverageVelocity */
  float mostbound_pos[3];         /* ComovingMostBoundPosition */
  float mostbound_vel[3];         /* PhysicalMostBoundVelocity */
  float specific_potential;       /* SpecificSelfPotentialEnergy */
  float specific_kinetic;         /* SpecificSelfKineticEnergy */
  float specific_angmom[3];       /* SpecificAngularMomentum */
  int64_t nbound_type[6];         /* NboundType */
  float mbound_type[6];           /* MboundType */
  int32_t iterations;             /* passes of the unbinding loop */
  int32_t disrupted;              /* 1 if the disruption branch was taken */
  int32_t converged;              /* 1 if the loop ended by convergence */
  int32_t too_few;                /* 1 if n < MinNumPartOfSub (death is recorded) */
  int64_t evaluations;            /* target potentials evaluated, all passes */
  int64_t interactions;           /* walk contributions summed, all passes */
  int64_t random_splits;          /* sub-resolution cells split at random (drand48), all passes */
} hbto_result;

/* Unbind one subhalo.
 *   n particles, arrays indexed by input position: id[n], pos[3n] (comoving,
 *   xyz per particle), vel[3n] (physical), mass[n], type[n] (0..5; may be NULL).
 *   *st: the subhalo's frame and most-bound record on entry.  Position 0
 *   holds the previous most-bound particle; when sampling applies
 *   (max_sample_size>0 && n>max_sample_size) the caller has already applied the
 *   reference's random_shuffle (see hbto_reference_shuffle) and st->mostbound_id
 *   names the particle that was at position 0 before it.
 * Outputs: order[n] -- output position i holds input particle order[i]
 *   (the reference's permuted Particles vector); energy[n] -- the binding energy
 *   held for output position i (the reference keeps the first nbound of these as
 *   Subhalo_t::Energies); *res.
 * nthreads: OpenMP threads for the particle loops (<=0: runtime default).
 * Returns 0 on success. */
int hbto_unbind(const hbto_params *par, int64_t n, const int64_t *id, const float *pos,
                const float *vel, const float *mass, const int32_t *type, const hbto_state *st,
                int64_t *order, float *energy, hbto_result *res, int nthreads);

/* Unbind nsub independent subhalos (particles of subhalo s at offsets
 * [off[s], off[s+1])), halo-parallel with schedule(dynamic,1) as in
 * SubhaloSnapshot_t::RefineParticles (src/subhalo_unbind.cpp:495-503).
 * st[nsub] as for hbto_unbind.  order[] holds positions local to each
 * subhalo.  drand48 state is shared between threads, as in the reference. */
int hbto_unbind_batch(const hbto_params *par, int64_t nsub, const int64_t *off, const int64_t *id,
                      const float *pos, const float *vel, const float *mass, const int32_t *type,
                      const hbto_state *st, int64_t *order, float *energy, hbto_result *res,
                      int nthreads);

/* One full-iteration energy pass: a tree over all n particles and, for every
 * particle, BindingEnergy(x, v, ref_pos, ref_vel, m) including the self-term
 * cancellation (the first pass of the loop, src/subhalo_unbind.cpp:333-354).
 * potential[n] (double, may be NULL) receives EvaluatePotential's value. */
int hbto_binding_energies(const hbto_params *par, int64_t n, const float *pos, const float *vel,
                          const float *mass, const float ref_pos[3], const float ref_vel[3],
                          float *energy, double *potential, int64_t *interactions, int nthreads);

/* EvaluatePotential (src/gravity_tree.cpp:79-164) of the particles
 * targets[0..ntarget) (indices into pos/mass) from one tree over all n
 * particles, self term cancelled, at each of ntheta opening angles (the tree is
 * built once): potential[k*ntarget + j] for open_angles[k]; interactions[k]
 * (may be NULL) counts the contributions summed.  par->open_angle is unused.
 * Returns 0, or 1 for a target out of range. */
int hbto_tree_potentials(const hbto_params *par, int64_t n, const float *pos, const float *mass,
                         int64_t ntarget, const int64_t *targets, int32_t ntheta,
                         const double *open_angles, double *potential, int64_t *interactions,
                         int nthreads);

/* The reference's Hoare-style split of an energy list
 * (PartitionBindingEnergy, src/subhalo_unbind.cpp:21-58): permutes E[] and
 * idx[] in place and returns the number of entries kept in front. */
int64_t hbto_partition(float *E, int64_t *idx, int64_t len);

/* Seed glibc's drand48 stream, which the tree build consumes for particles
 * closer than TreeNodeResolution (src/oct_tree.tpp:112-123). */
void hbto_srand48(long seed);

/* Fill perm[0..n) with the permutation that srand(seed) followed by
 * std::random_shuffle applies to an n-element vector
 * (src/subhalo_unbind.cpp:302): perm[i] = original index now at i. */
void hbto_reference_shuffle(int64_t n, unsigned seed, int64_t *perm);

/* Post-unbinding properties of a subhalo (Subhalo_t members written by
 * CalculateProfileProperties, src/subhalo.cpp:242-335, and CalculateShape,
 * :337-398). */
typedef struct {
  float rmax_comoving, vmax_physical, last_max_vmax_physical;
  int32_t snapshot_of_last_max_vmax;
  float r2sigma_comoving, rhalf_comoving, r200crit_comoving, m200crit;
  float inertial_tensor[6], inertial_tensor_weighted[6];
} hbto_props;

/* CalculateProfileProperties + CalculateShape (src/subhalo.cpp:242-398) of a
 * subhalo whose bound particles, most-bound first, are pos[3*nbound] and
 * mass[nbound]; cen is ComovingMostBoundPosition, mbound its Mbound; the
 * epoch is snapshot `snapshot_index` with G, Hz, a from par.  Ties in radius
 * keep the given order (the reference's std::sort leaves them unspecified). */
int hbto_subhalo_properties(const hbto_params *par, int64_t nbound, const float *pos,
                            const float *mass, const float cen[3], float mbound,
                            float last_max_vmax, int32_t last_snap, int32_t snapshot_index,
                            hbto_props *out);

/* Core of a subhalo as the merging step sees it (SubHelper_t,
 * src/subhalo_merge.cpp:14-26): mean position and velocity of its first
 * min(Nbound, 20) particles and their dispersions. */
typedef struct {
  float pos[3];
  float sigma_r;
  float vel[3];
  float sigma_v;
} hbto_core;

/* FillCores and DetectTraps of SubhaloSnapshot_t::MergeSubhalos
 * (src/subhalo_merge.cpp:30-180): subhalo s holds particles
 * [list_off[s], list_off[s+1]) of pos/vel/mass, bound first; host[s] its
 * HostTrackId (-1: none); mb_pos/mb_vel its ComovingMostBoundPosition and
 * PhysicalMostBoundVelocity.  sink[s] is SinkTrackId on entry (-1: not yet
 * trapped) and on exit; a subhalo trapped now gets sink_snap[s] = isnap (other
 * entries are left alone), and its host merged[host] = 1 when the subhalo has
 * Nbound > 1.  cores may be NULL.  Returns -1 if a host chain is longer than
 * nsub (a cycle). */
int hbto_merge_detect(const hbto_params *par, int64_t nsub, const int64_t *list_off,
                      const float *pos, const float *vel, const float *mass,
                      const int64_t *nbound, const int64_t *host, const float *mb_pos,
                      const float *mb_vel, int32_t isnap, int64_t *sink, int32_t *sink_snap,
                      int32_t *merged, hbto_core *cores);

/* Particle-ID -> index tables (src/hash.h:47-112, src/hash.tpp, src/hash_remote.tpp).
 * Fill a table with the pairs (keys[i], values[i]), i < n (KeyList_t::GetKey and
 * ::GetIndex), then look up every query: out[j] = GetIndex(queries[j]), or
 * null_index when the key is absent.
 *   flat = 0: MappedIndexTable_t -- pairs sorted by key, binary search; a
 *             negative key is absent (hash.tpp:18-55);
 *   flat = 1: FlatIndexTable_t -- a dense array over [KeyMin, KeyMax]
 *             (hash.tpp:59-109).
 * Duplicate keys are not defined by the reference (std::sort is not stable,
 * and the flat fill writes in parallel); here the first pair in input order
 * wins for the mapped table and the last for the flat one. */
int hbto_index_lookup(int flat, const int64_t *keys, const int64_t *values, int64_t n,
                      int64_t null_index, const int64_t *queries, int64_t m, int64_t *out);

#ifdef __cplusplus
}
#endif
#endif
