/* ref_driver.cpp -- harness around the reference's own Subhalo_t::Unbind.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled (by oracle/Makefile, target `ref`)
 * together with the unmodified reference sources where they lie, into
 * oracle/_ref/libhbt_ref.so, which is never committed.  It exports the
 * entry points of oracle/hbt_oracle.h with the prefix ref_, so that the C
 * restatement can be pinned against the reference on identical inputs and
 * the reference can be timed as the CPU baseline.
 *
 * Differences from the hbto_ entry points:
 *   - ref_unbind/ref_unbind_batch take the particles in their order BEFORE
 *     the sampling shuffle (position 0 = previous most-bound) plus the seed
 *     for srand(); the reference shuffles them itself
 *     (src/subhalo_unbind.cpp:302).
 *   - iterations/evaluations/interactions are not available (left 0).
 */
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "config_parser.h"
#include "datatypes.h"
#include "gravity_tree.h"
#include "snapshot.h"
#include "subhalo.h"
#include "hash.h"
#include "hash_remote.tpp"

#include "../hbt_oracle.h"

namespace {

/* The reference's configuration as ParseConfigFile leaves it
 * (src/config_parser.cpp:95-103), for the unbinding subset. */
void setup(const hbto_params *p)
{
  HBTConfig.SofteningHalo = p->softening;
  HBTConfig.TreeNodeOpenAngle = p->open_angle;
  HBTConfig.BoundMassPrecision = p->bound_mass_precision;
  HBTConfig.MinNumPartOfSub = (int)p->min_num_part;
  HBTConfig.MaxSampleSizeOfPotentialEstimate = p->max_sample_size;
  HBTConfig.RefineMostboundParticle = p->refine_mostbound != 0;
  HBTConfig.PeriodicBoundaryOn = p->periodic != 0;
  HBTConfig.BoxSize = p->box_size;
  PhysicalConst::G = p->G;
  HBTConfig.BoxHalf = HBTConfig.BoxSize / 2.;
  HBTConfig.TreeNodeResolution = HBTConfig.SofteningHalo * 0.1;
  HBTConfig.TreeNodeResolutionHalf = HBTConfig.TreeNodeResolution / 2.;
  HBTConfig.TreeNodeOpenAngleSquare = HBTConfig.TreeNodeOpenAngle * HBTConfig.TreeNodeOpenAngle;
}

/* The snapshot handed to Unbind: only Cosmology and the snapshot index are read. */
class Epoch_t : public Snapshot_t
{
public:
  Epoch_t(const hbto_params *p)
  {
    Cosmology.ScaleFactor = p->scale_factor;
    Cosmology.Hz = p->hubble;
    Cosmology.OmegaM0 = 0.3;
    Cosmology.OmegaLambda0 = 0.7;
    Cosmology.OmegaZ = 0.3;
    SnapshotIndex = 1;
    SnapshotId = 1;
  }
  HBTInt size() const { return 0; }
  const HBTxyz &GetComovingPosition(const HBTInt) const { return dummy; }
  const HBTxyz &GetPhysicalVelocity(const HBTInt) const { return dummy; }
  HBTReal GetMass(const HBTInt) const { return 0; }

private:
  HBTxyz dummy{{0, 0, 0}};
};

/* A plain particle array viewed as a Snapshot_t, for the tree-only entry. */
class ArraySnapshot_t : public Snapshot_t
{
public:
  ArraySnapshot_t(const hbto_params *p, int64_t n, const float *pos, const float *vel,
                  const float *mass)
      : P(n), V(n), M(mass, mass + n)
  {
    Cosmology.ScaleFactor = p->scale_factor;
    Cosmology.Hz = p->hubble;
    for (int64_t i = 0; i < n; i++)
      for (int j = 0; j < 3; j++) {
        P[i][j] = pos[3 * i + j];
        V[i][j] = vel[3 * i + j];
      }
  }
  HBTInt size() const { return P.size(); }
  const HBTxyz &GetComovingPosition(const HBTInt i) const { return P[i]; }
  const HBTxyz &GetPhysicalVelocity(const HBTInt i) const { return V[i]; }
  HBTReal GetMass(const HBTInt i) const { return M[i]; }
  std::vector<HBTxyz> P, V;
  std::vector<HBTReal> M;
};

void fill_subhalo(Subhalo_t &sub, int64_t n, const int64_t *id, const float *pos, const float *vel,
                  const float *mass, const int32_t *type, const hbto_state *st)
{
  sub.Particles.resize(n);
  for (int64_t i = 0; i < n; i++) {
    Particle_t &p = sub.Particles[i];
    p.Id = id[i];
    for (int j = 0; j < 3; j++) {
      p.ComovingPosition[j] = pos[3 * i + j];
      p.PhysicalVelocity[j] = vel[3 * i + j];
    }
    p.Mass = mass[i];
    p.Type = (ParticleType_t)(type ? type[i] : 1);
  }
  sub.Nbound = n;
  for (int j = 0; j < 3; j++) {
    sub.ComovingAveragePosition[j] = st->ref_pos[j];
    sub.PhysicalAverageVelocity[j] = st->ref_vel[j];
    sub.ComovingMostBoundPosition[j] = st->mostbound_pos[j];
    sub.PhysicalMostBoundVelocity[j] = st->mostbound_vel[j];
  }
}

/* Output ids are mapped back to input positions through the caller's id list
 * (ids are unique in every input the tests use). */
void read_subhalo(const Subhalo_t &sub, int64_t n, const int64_t *id_sorted_pos,
                  const int64_t *id_sorted, int64_t *order, float *energy, hbto_result *res,
                  int64_t nin)
{
  std::memset(res, 0, sizeof(*res));
  res->nbound = sub.Nbound;
  res->mbound = sub.Mbound;
  for (int j = 0; j < 3; j++) {
    res->ref_pos[j] = sub.ComovingAveragePosition[j];
    res->ref_vel[j] = sub.PhysicalAverageVelocity[j];
    res->mostbound_pos[j] = sub.ComovingMostBoundPosition[j];
    res->mostbound_vel[j] = sub.PhysicalMostBoundVelocity[j];
    res->specific_angmom[j] = sub.SpecificAngularMomentum[j];
  }
  res->specific_potential = sub.SpecificSelfPotentialEnergy;
  res->specific_kinetic = sub.SpecificSelfKineticEnergy;
  for (int k = 0; k < 6; k++) {
    res->nbound_type[k] = sub.NboundType[k];
    res->mbound_type[k] = sub.MboundType[k];
  }
  for (int64_t i = 0; i < n; i++) {
    int64_t key = sub.Particles[i].Id;
    const int64_t *it = std::lower_bound(id_sorted, id_sorted + nin, key);
    order[i] = (it != id_sorted + nin && *it == key) ? id_sorted_pos[it - id_sorted] : -1;
    energy[i] = i < (int64_t)sub.Energies.size() ? sub.Energies[i] : NAN;
  }
}

void sorted_ids(int64_t n, const int64_t *id, std::vector<int64_t> &ids, std::vector<int64_t> &pos)
{
  std::vector<std::pair<int64_t, int64_t>> v(n);
  for (int64_t i = 0; i < n; i++) v[i] = std::make_pair(id[i], i);
  std::sort(v.begin(), v.end());
  ids.resize(n);
  pos.resize(n);
  for (int64_t i = 0; i < n; i++) {
    ids[i] = v[i].first;
    pos[i] = v[i].second;
  }
}

/* The (key, index) pairs handed to IndexTable_t::Fill (src/hash.h:10-17). */
class ArrayKeyList_t : public KeyList_t<HBTInt, HBTInt>
{
  const int64_t *keys_, *values_;
  HBTInt n_;

public:
  ArrayKeyList_t(const int64_t *k, const int64_t *v, int64_t n) : keys_(k), values_(v), n_(n) {}
  HBTInt GetKey(const HBTInt i) const { return keys_[i]; }
  HBTInt GetIndex(const HBTInt i) const { return values_[i]; }
  HBTInt size() const { return n_; }
};

/* A list of particles as GetIndices takes it: elements with an Id field. */
struct IdOnly_t {
  HBTInt Id;
};

/* A SubhaloSnapshot_t holding only what MergeSubhalos reads: the subhaloes,
 * the halo membership table, the snapshot index and the cosmology. */
class MergeSnap_t : public SubhaloSnapshot_t
{
public:
  MergeSnap_t(const hbto_params *p, int isnap)
  {
    Cosmology.ScaleFactor = p->scale_factor;
    Cosmology.Hz = p->hubble;
    Cosmology.OmegaM0 = 0.3;
    Cosmology.OmegaLambda0 = 0.7;
    Cosmology.OmegaZ = 0.3;
    SnapshotIndex = isnap;
    SnapshotId = isnap;
  }
};

}  // namespace

/* Stand-ins for the SubhaloSnapshot_t members whose own definitions sit in
 * files this harness does not compile (they need MPI and HDF5).  The HDF5
 * type set-up is never used here.  GlueHeadNests / UnglueHeadNests restate
 * src/subhalo_tracking.cpp:843-874: while merging, the other top-level
 * subhaloes of a halo join its central's nest, and leave it afterwards. */
void SubhaloSnapshot_t::BuildHDFDataType() {}
herr_t H5Tclose(hid_t) { return 0; }
void SubhaloSnapshot_t::GlueHeadNests()
{
#pragma omp single
  {
    RootNestSize.resize(MemberTable.SubGroups.size());
    for (HBTInt h = 0; h < (HBTInt)RootNestSize.size(); h++) {
      auto &group = MemberTable.SubGroups[h];
      if (group.size() == 0) {
        RootNestSize[h] = 0;
        continue;
      }
      auto &nest = Subhalos[group[0]].NestedSubhalos;
      RootNestSize[h] = nest.size();
      auto &heads = MemberTable.SubGroupsOfHeads[h];
      nest.insert(nest.end(), heads.begin() + 1, heads.end());
    }
  }
}
void SubhaloSnapshot_t::UnglueHeadNests()
{
#pragma omp single
  {
    for (HBTInt h = 0; h < (HBTInt)RootNestSize.size(); h++) {
      auto &group = MemberTable.SubGroups[h];
      if (group.size()) Subhalos[group[0]].NestedSubhalos.resize(RootNestSize[h]);
    }
    RootNestSize.clear();
  }
}

extern "C" {

/* RecursiveUnbind over a forest of subhaloes, then TruncateSource on all
 * (src/subhalo_unbind.cpp:432-458, the non-INCLUSIVE_MASS branch of
 * RefineParticles, :475-515): subhalo s starts with its own particles
 * own[list_off[s] .. list_off[s+1]), the Nbound of the last snapshot
 * (nbound_prev[s]; <= 1 makes it an orphan) and its nested subhaloes
 * nest_idx[nest_off[s] .. nest_off[s+1]); roots[] are unbound in order.
 * Output: each subhalo's final particle list as positions into the input
 * arrays (out_off[nsub+1], out_pos[out_capacity]; a tail handed to a host
 * can stay in the satellite's truncated list too), and its results. */
int ref_recursive_unbind(const hbto_params *par, double relax_factor, int64_t nsub,
                         const int64_t *list_off, const int64_t *id, const float *pos,
                         const float *vel, const float *mass, const int32_t *type,
                         const int64_t *nbound_prev, const hbto_state *st,
                         const int64_t *nest_off, const int64_t *nest_idx, int64_t nroot,
                         const int64_t *roots, int64_t *out_off, int64_t *out_pos,
                         int64_t out_capacity, hbto_result *res)
{
  setup(par);
  HBTConfig.SourceSubRelaxFactor = relax_factor;
  omp_set_num_threads(1);
  omp_set_max_active_levels(1);
  Epoch_t epoch(par);
  SubhaloList_t subs(nsub);
  for (int64_t s = 0; s < nsub; s++) {
    const int64_t o = list_off[s], n = list_off[s + 1] - o;
    fill_subhalo(subs[s], n, id + o, pos + 3 * o, vel + 3 * o, mass + o, type ? type + o : nullptr,
                 st + s);
    subs[s].Nbound = nbound_prev[s];
    subs[s].NestedSubhalos.assign(nest_idx + nest_off[s], nest_idx + nest_off[s + 1]);
  }
  srand(0);
  for (int64_t r = 0; r < nroot; r++) subs[roots[r]].RecursiveUnbind(subs, epoch);
  for (int64_t s = 0; s < nsub; s++) subs[s].TruncateSource();
  const int64_t ntot = list_off[nsub];
  std::vector<int64_t> ids, ipos;
  sorted_ids(ntot, id, ids, ipos);
  out_off[0] = 0;
  for (int64_t s = 0; s < nsub; s++) {
    const int64_t n = subs[s].Particles.size();
    if (out_off[s] + n > out_capacity) return -1;  // lists may share particles: ask for more
    std::vector<float> en(n);
    read_subhalo(subs[s], n, ipos.data(), ids.data(), out_pos + out_off[s], en.data(), res + s,
                 ntot);
    out_off[s + 1] = out_off[s] + n;
  }
  return 0;
}

/* Unbind, then the reference's CalculateProfileProperties and CalculateShape
 * (src/subhalo.cpp:242-398) on the result; last_max_vmax and last_snap are
 * the subhalo's LastMaxVmaxPhysical and SnapshotIndexOfLastMaxVmax before the
 * call (the epoch is snapshot 1). */
int ref_unbind_properties(const hbto_params *par, int64_t n, const int64_t *id, const float *pos,
                          const float *vel, const float *mass, const int32_t *type,
                          const hbto_state *st, float last_max_vmax, int32_t last_snap,
                          int64_t *order, float *energy, hbto_result *res, hbto_props *props)
{
  setup(par);
  omp_set_num_threads(1);
  omp_set_max_active_levels(1);
  PhysicalConst::H0 = 100.;
  Epoch_t epoch(par);
  Subhalo_t sub;
  fill_subhalo(sub, n, id, pos, vel, mass, type, st);
  sub.LastMaxVmaxPhysical = last_max_vmax;
  sub.SnapshotIndexOfLastMaxVmax = last_snap;
  sub.BoundM200Crit = 0.f;  // left as is when no radius qualifies (snapshot.cpp:270-280)
  sub.BoundR200CritComoving = 0.f;
  srand(0);
  sub.Unbind(epoch);
  sub.CalculateProfileProperties(epoch);
  sub.CalculateShape();
  std::vector<int64_t> ids, ipos;
  sorted_ids(n, id, ids, ipos);
  read_subhalo(sub, n, ipos.data(), ids.data(), order, energy, res, n);
  props->rmax_comoving = sub.RmaxComoving;
  props->vmax_physical = sub.VmaxPhysical;
  props->last_max_vmax_physical = sub.LastMaxVmaxPhysical;
  props->snapshot_of_last_max_vmax = sub.SnapshotIndexOfLastMaxVmax;
  props->r2sigma_comoving = sub.R2SigmaComoving;
  props->rhalf_comoving = sub.RHalfComoving;
  props->r200crit_comoving = sub.BoundR200CritComoving;
  props->m200crit = sub.BoundM200Crit;
  for (int k = 0; k < 6; k++) {
    props->inertial_tensor[k] = sub.InertialTensor[k];
    props->inertial_tensor_weighted[k] = sub.InertialTensorWeighted[k];
  }
  return 0;
}

/* The reference's own tables: Fill, then GetIndex per query (src/hash.tpp). */
int ref_index_lookup(int flat, const int64_t *keys, const int64_t *values, int64_t n,
                     int64_t null_index, const int64_t *queries, int64_t m, int64_t *out)
{
  ArrayKeyList_t list(keys, values, n);
  if (flat) {
    FlatIndexTable_t<HBTInt, HBTInt> table;
    table.Fill(list, null_index);
    for (int64_t j = 0; j < m; j++) out[j] = table.GetIndex(queries[j]);
  } else {
    MappedIndexTable_t<HBTInt, HBTInt> table;
    table.Fill(list, null_index);
    for (int64_t j = 0; j < m; j++) out[j] = table.GetIndex(queries[j]);
  }
  return 0;
}

/* The batch form, GetIndices (src/hash_remote.tpp:5-99); the mapped table's
 * recursive search expects the queries in ascending order. */
int ref_index_lookup_batch(int flat, const int64_t *keys, const int64_t *values, int64_t n,
                           int64_t null_index, const int64_t *queries, int64_t m, int64_t *out)
{
  ArrayKeyList_t list(keys, values, n);
  std::vector<IdOnly_t> parts(m);
  for (int64_t j = 0; j < m; j++) parts[j].Id = queries[j];
  if (flat) {
    FlatIndexTable_t<HBTInt, HBTInt> table;
    table.Fill(list, null_index);
    table.GetIndices(parts);
  } else {
    MappedIndexTable_t<HBTInt, HBTInt> table;
    table.Fill(list, null_index);
    table.GetIndices(parts);
  }
  for (int64_t j = 0; j < m; j++) out[j] = parts[j].Id;
  return 0;
}

int ref_unbind(const hbto_params *par, int64_t n, const int64_t *id, const float *pos,
               const float *vel, const float *mass, const int32_t *type, const hbto_state *st,
               int64_t *order, float *energy, hbto_result *res, int nthreads,
               unsigned shuffle_seed)
{
  setup(par);
  if (nthreads > 0) omp_set_num_threads(nthreads);
  omp_set_max_active_levels(1);
  Epoch_t epoch(par);
  Subhalo_t sub;
  fill_subhalo(sub, n, id, pos, vel, mass, type, st);
  srand(shuffle_seed);
  sub.Unbind(epoch);
  std::vector<int64_t> ids, ipos;
  sorted_ids(n, id, ids, ipos);
  read_subhalo(sub, n, ipos.data(), ids.data(), order, energy, res, n);
  res->too_few = n < par->min_num_part;
  res->disrupted = (n >= 2 && sub.Nbound == 1);
  res->converged = (n >= 2 && !res->disrupted);
  return 0;
}

int ref_unbind_batch(const hbto_params *par, int64_t nsub, const int64_t *off, const int64_t *id,
                     const float *pos, const float *vel, const float *mass, const int32_t *type,
                     const hbto_state *st, int64_t *order, float *energy, hbto_result *res,
                     int nthreads, unsigned shuffle_seed)
{
  setup(par);
  if (nthreads > 0) omp_set_num_threads(nthreads);
  omp_set_max_active_levels(1);
  Epoch_t epoch(par);
  std::vector<Subhalo_t> subs(nsub);
  for (int64_t s = 0; s < nsub; s++) {
    const int64_t o = off[s];
    fill_subhalo(subs[s], off[s + 1] - o, id + o, pos + 3 * o, vel + 3 * o, mass + o,
                 type ? type + o : nullptr, st + s);
  }
  srand(shuffle_seed);
  /* the field-subhalo loop of SubhaloSnapshot_t::RefineParticles
   * (src/subhalo_unbind.cpp:495-503) */
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t s = 0; s < nsub; s++) subs[s].Unbind(epoch);
  for (int64_t s = 0; s < nsub; s++) {
    const int64_t o = off[s], m = off[s + 1] - off[s];
    std::vector<int64_t> ids, ipos;
    sorted_ids(m, id + o, ids, ipos);
    read_subhalo(subs[s], m, ipos.data(), ids.data(), order + o, energy + o, res + s, m);
    res[s].too_few = m < par->min_num_part;
    res[s].disrupted = (m >= 2 && subs[s].Nbound == 1);
    res[s].converged = (m >= 2 && !res[s].disrupted);
  }
  return 0;
}

int ref_binding_energies(const hbto_params *par, int64_t n, const float *pos, const float *vel,
                         const float *mass, const float ref_pos[3], const float ref_vel[3],
                         float *energy, double *potential, int64_t *interactions, int nthreads)
{
  setup(par);
  if (nthreads > 0) omp_set_num_threads(nthreads);
  ArraySnapshot_t snap(par, n, pos, vel, mass);
  GravityTree_t tree;
  tree.Reserve(n);
  tree.Build(snap);
  HBTxyz rp, rv;
  for (int j = 0; j < 3; j++) {
    rp[j] = ref_pos[j];
    rv[j] = ref_vel[j];
  }
#pragma omp parallel for if (n > 100)
  for (int64_t i = 0; i < n; i++) {
    if (potential) potential[i] = tree.EvaluatePotential(snap.P[i], snap.M[i]);
    energy[i] = tree.BindingEnergy(snap.P[i], snap.V[i], rp, rv, snap.M[i]);
  }
  if (interactions) *interactions = 0;
  return 0;
}

void ref_srand48(long seed) { srand48(seed); }

/* SubhaloSnapshot_t::MergeSubhalos (src/subhalo_merge.cpp:187-220) with
 * MergeTrappedSubhalos on, at snapshot isnap, over subhaloes after their
 * unbinding: subhalo s holds the particles [list_off[s], list_off[s+1]) of
 * the arrays (bound first), Nbound nbound[s], frames st[s]
 * (ref_pos/ref_vel = ComovingAveragePosition/PhysicalAverageVelocity), nested
 * subhaloes nest_idx[nest_off[s]..), SinkTrackId sink_in[s] and
 * SnapshotIndexOfDeath death_in[s]; halo h has members
 * group_idx[group_off[h]..) (central first) and top-level subhaloes
 * heads_idx[heads_off[h]..) (central first).  Output per subhalo: the
 * particle Ids of its list (out_off, out_id), their energies where the
 * re-unbinding kept them (out_energy), SinkTrackId, SnapshotIndexOfDeath,
 * SnapshotIndexOfSink, and its results. */
int ref_merge_subhalos(const hbto_params *par, double relax_factor, int32_t isnap, int64_t nsub,
                       const int64_t *list_off, const int64_t *id, const float *pos,
                       const float *vel, const float *mass, const int32_t *type,
                       const int64_t *nbound, const hbto_state *st, const int64_t *nest_off,
                       const int64_t *nest_idx, int64_t nhalo, const int64_t *group_off,
                       const int64_t *group_idx, const int64_t *heads_off,
                       const int64_t *heads_idx, const int64_t *sink_in, const int32_t *death_in,
                       int64_t out_capacity, int64_t *out_off, int64_t *out_id,
                       float *out_energy, int64_t *sink_out, int32_t *death_out,
                       int32_t *sink_snap_out, hbto_result *res)
{
  setup(par);
  HBTConfig.SourceSubRelaxFactor = relax_factor;
  HBTConfig.MergeTrappedSubhalos = true;
  omp_set_num_threads(1);
  omp_set_max_active_levels(1);
  std::vector<HBTInt> members(group_idx, group_idx + group_off[nhalo]);
  std::vector<MemberShipTable_t::MemberList_t> views(nhalo);
  for (int64_t h = 0; h < nhalo; h++)
    views[h].Bind(group_off[h + 1] - group_off[h], members.data() + group_off[h]);
  MergeSnap_t snap(par, isnap);
  snap.Subhalos.resize(nsub);
  for (int64_t s = 0; s < nsub; s++) {
    Subhalo_t &sub = snap.Subhalos[s];
    const int64_t o = list_off[s], n = list_off[s + 1] - o;
    fill_subhalo(sub, n, id + o, pos + 3 * o, vel + 3 * o, mass + o, type ? type + o : nullptr,
                 st + s);
    sub.Nbound = nbound[s];
    sub.NestedSubhalos.assign(nest_idx + nest_off[s], nest_idx + nest_off[s + 1]);
    sub.SinkTrackId = sink_in[s];
    sub.SnapshotIndexOfDeath = death_in[s];
    sub.CountParticles();
  }
  snap.MemberTable.SubGroups.Bind(nhalo, views.data());
  snap.MemberTable.SubGroupsOfHeads.resize(nhalo);
  for (int64_t h = 0; h < nhalo; h++)
    snap.MemberTable.SubGroupsOfHeads[h].assign(heads_idx + heads_off[h],
                                                heads_idx + heads_off[h + 1]);
  srand(0);
  snap.MergeSubhalos();
  const int64_t ntot = list_off[nsub];
  std::vector<int64_t> ids, ipos;
  sorted_ids(ntot, id, ids, ipos);
  out_off[0] = 0;
  for (int64_t s = 0; s < nsub; s++) {
    const Subhalo_t &sub = snap.Subhalos[s];
    const int64_t n = sub.Particles.size();
    if (out_off[s] + n > out_capacity) return -1;
    std::vector<int64_t> order(n);
    read_subhalo(sub, n, ipos.data(), ids.data(), order.data(), out_energy + out_off[s], res + s,
                 ntot);
    for (int64_t i = 0; i < n; i++) out_id[out_off[s] + i] = sub.Particles[i].Id;
    sink_out[s] = sub.SinkTrackId;
    death_out[s] = sub.SnapshotIndexOfDeath;
    sink_snap_out[s] = sub.SnapshotIndexOfSink;
    out_off[s + 1] = out_off[s] + n;
  }
  return 0;
}

}  // extern "C"
