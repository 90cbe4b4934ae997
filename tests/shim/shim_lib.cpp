// shim_lib.cpp -- test harness of include/hbtu_subhalo.hpp.
//
// Stand-ins for HBT+'s Particle_t / Subhalo_t / Snapshot_t with the member
// names and types of src/snapshot.h:51-72 and src/subhalo.h:24-146 (HBT_INT8,
// float HBTReal), so the shim is exercised exactly as the reference would use
// it.  shim_unbind() builds one subhalo, calls hbtu::UnbindGPU and reports the
// subhalo as Unbind leaves it.
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "hbtu_subhalo.hpp"

namespace mock {
typedef std::array<float, 3> HBTxyz;
struct Particle_t {
  long Id;
  HBTxyz ComovingPosition;
  HBTxyz PhysicalVelocity;
  float Mass;
  int Type;
  long Row = -1;  // harness only: the input row this particle came from
};
struct Subhalo_t {
  long TrackId = 0, Nbound = 0;
  float Mbound = 0;
  long NboundType[6] = {0};
  float MboundType[6] = {0};
  int SnapshotIndexOfDeath = -1, SnapshotIndexOfSink = -1;
  float SpecificSelfPotentialEnergy = 0, SpecificSelfKineticEnergy = 0;
  float SpecificAngularMomentum[3] = {0, 0, 0};
  HBTxyz ComovingAveragePosition, PhysicalAverageVelocity, ComovingMostBoundPosition,
      PhysicalMostBoundVelocity;
  long SinkTrackId = -1;
  float RmaxComoving = 0, VmaxPhysical = 0, LastMaxVmaxPhysical = 0;
  int SnapshotIndexOfLastMaxVmax = -1;
  float R2SigmaComoving = 0, RHalfComoving = 0, BoundR200CritComoving = 0, BoundM200Crit = 0;
  float InertialTensor[6] = {0}, InertialTensorWeighted[6] = {0};
  std::vector<Particle_t> Particles;
  std::vector<long> NestedSubhalos;
  bool IsTrapped() { return SinkTrackId != -1; }
  bool IsAlive() { return SnapshotIndexOfDeath == -1; }
  void CountParticles()  // Subhalo_t::CountParticleTypes (src/subhalo.cpp:400-444), serial
  {
    for (int t = 0; t < 6; t++) {
      NboundType[t] = 0;
      MboundType[t] = 0.f;
    }
    for (long i = 0; i < Nbound && i < (long)Particles.size(); i++) {
      if (Particles[i].Id == -1) continue;
      NboundType[Particles[i].Type]++;
      MboundType[Particles[i].Type] += Particles[i].Mass;
    }
  }
};
struct Snapshot_t {
  int index = 7;
  int GetSnapshotIndex() const { return index; }
};
// MemberShipTable_t (src/subhalo.h:148-185): SubGroups[-1] are the field
// subhaloes, SubGroups[0 .. size()) the haloes' members (central first).
struct GroupView {
  std::vector<std::vector<long>> g;  // g[0]: the field
  const std::vector<long> &operator[](long i) const { return g[i + 1]; }
  size_t size() const { return g.size() - 1; }
};
struct MemberShipTable_t {
  GroupView SubGroups;
  std::vector<std::vector<long>> SubGroupsOfHeads;
  std::vector<long> AllMembers;
};
struct SubhaloSnapshot_t : Snapshot_t {
  std::vector<Subhalo_t> Subhalos;
  MemberShipTable_t MemberTable;
};
}  // namespace mock

namespace {

// Subhaloes s of the harness: particles of rows list_off[s] .. list_off[s+1].
void build_subhaloes(std::vector<mock::Subhalo_t> &subs, int64_t nsub, const int64_t *list_off,
                     const int64_t *id, const float *pos, const float *vel, const float *mass,
                     const int32_t *type, const int64_t *nbound, const float *ref_pos,
                     const float *ref_vel, const float *mb_pos, const float *mb_vel,
                     const int64_t *nest_off, const int64_t *nest_idx)
{
  subs.assign(nsub, mock::Subhalo_t());
  for (int64_t s = 0; s < nsub; s++) {
    mock::Subhalo_t &sub = subs[s];
    for (int64_t i = list_off[s]; i < list_off[s + 1]; i++) {
      mock::Particle_t q;
      q.Id = id[i];
      for (int j = 0; j < 3; j++) {
        q.ComovingPosition[j] = pos[3 * i + j];
        q.PhysicalVelocity[j] = vel[3 * i + j];
      }
      q.Mass = mass[i];
      q.Type = type ? type[i] : 1;
      q.Row = i;
      sub.Particles.push_back(q);
    }
    sub.Nbound = nbound[s];
    for (int j = 0; j < 3; j++) {
      sub.ComovingAveragePosition[j] = ref_pos[3 * s + j];
      sub.PhysicalAverageVelocity[j] = ref_vel[3 * s + j];
      sub.ComovingMostBoundPosition[j] = mb_pos[3 * s + j];
      sub.PhysicalMostBoundVelocity[j] = mb_vel[3 * s + j];
    }
    for (int64_t k = nest_off[s]; k < nest_off[s + 1]; k++) sub.NestedSubhalos.push_back(nest_idx[k]);
  }
}

std::vector<std::vector<long>> lists_of(int64_t n, const int64_t *off, const int64_t *idx)
{
  std::vector<std::vector<long>> out(n);
  for (int64_t i = 0; i < n; i++)
    for (int64_t k = off[i]; k < off[i + 1]; k++) out[i].push_back(idx[k]);
  return out;
}

}  // namespace

extern "C" int shim_unbind(hbtu_handle *h, const hbtu_params *par, int64_t n, const int64_t *id,
                           const float *pos, const float *vel, const float *mass,
                           const int32_t *type, const hbtu_state *st, int64_t *out_id,
                           float *out_energy, hbtu_result *out, int32_t *death, int32_t via_batch)
{
  mock::Subhalo_t s;
  s.Particles.resize(n);
  for (int64_t i = 0; i < n; i++) {
    s.Particles[i].Id = id[i];
    for (int j = 0; j < 3; j++) {
      s.Particles[i].ComovingPosition[j] = pos[3 * i + j];
      s.Particles[i].PhysicalVelocity[j] = vel[3 * i + j];
    }
    s.Particles[i].Mass = mass[i];
    s.Particles[i].Type = type ? type[i] : 1;
  }
  for (int j = 0; j < 3; j++) {
    s.ComovingAveragePosition[j] = st->ref_pos[j];
    s.PhysicalAverageVelocity[j] = st->ref_vel[j];
    s.ComovingMostBoundPosition[j] = st->mostbound_pos[j];
    s.PhysicalMostBoundVelocity[j] = st->mostbound_vel[j];
  }
  mock::Snapshot_t epoch;
  std::vector<float> energies;
  hbtu_status rc;
  if (via_batch) {  // the same subhalo through the batch form
    std::vector<mock::Subhalo_t> one(1, s);
    std::vector<std::vector<float>> en;
    rc = hbtu::UnbindBatchGPU(h, *par, one, {0}, epoch, &en);
    s = one[0];
    energies = en[0];
  } else {
    rc = hbtu::UnbindGPU(h, *par, s, epoch, &energies);
  }
  if (rc != HBTU_OK && rc != HBTU_ERR_NOT_CONVERGED) return rc;
  for (int64_t i = 0; i < n; i++) out_id[i] = s.Particles[i].Id;
  for (size_t i = 0; i < energies.size(); i++) out_energy[i] = energies[i];
  std::memset(out, 0, sizeof(*out));
  out->nbound = s.Nbound;
  out->mbound = s.Mbound;
  for (int j = 0; j < 3; j++) {
    out->ref_pos[j] = s.ComovingAveragePosition[j];
    out->ref_vel[j] = s.PhysicalAverageVelocity[j];
    out->mostbound_pos[j] = s.ComovingMostBoundPosition[j];
    out->mostbound_vel[j] = s.PhysicalMostBoundVelocity[j];
  }
  for (int t = 0; t < 6; t++) out->nbound_type[t] = s.NboundType[t];
  *death = s.SnapshotIndexOfDeath;
  return rc;
}

// One subhalo as Unbind leaves it (particles bound first), through
// hbtu::PropertiesGPU at snapshot 7; the property members come back in `out`
// (the layout of hbtu_props).
extern "C" int shim_properties(hbtu_handle *h, int64_t n, const int64_t *id, const float *pos,
                               const float *mass, int64_t nbound, float mbound,
                               const float *mostbound_pos, float last_max_vmax,
                               int32_t last_snap, hbtu_props *out)
{
  std::vector<mock::Subhalo_t> subs(1);
  mock::Subhalo_t &s = subs[0];
  s.Particles.resize(n);
  for (int64_t i = 0; i < n; i++) {
    s.Particles[i].Id = id[i];
    for (int j = 0; j < 3; j++) {
      s.Particles[i].ComovingPosition[j] = pos[3 * i + j];
      s.Particles[i].PhysicalVelocity[j] = 0.f;
    }
    s.Particles[i].Mass = mass[i];
    s.Particles[i].Type = 1;
  }
  s.Nbound = nbound;
  s.Mbound = mbound;
  for (int j = 0; j < 3; j++) s.ComovingMostBoundPosition[j] = mostbound_pos[j];
  s.LastMaxVmaxPhysical = last_max_vmax;
  s.SnapshotIndexOfLastMaxVmax = last_snap;
  mock::Snapshot_t epoch;
  const hbtu_status rc = hbtu::PropertiesGPU(h, subs, {0}, epoch);
  if (rc != HBTU_OK) return rc;
  out->rmax_comoving = s.RmaxComoving;
  out->vmax_physical = s.VmaxPhysical;
  out->last_max_vmax_physical = s.LastMaxVmaxPhysical;
  out->snapshot_of_last_max_vmax = s.SnapshotIndexOfLastMaxVmax;
  out->r2sigma_comoving = s.R2SigmaComoving;
  out->rhalf_comoving = s.RHalfComoving;
  out->r200crit_comoving = s.BoundR200CritComoving;
  out->m200crit = s.BoundM200Crit;
  for (int t = 0; t < 6; t++) {
    out->inertial_tensor[t] = s.InertialTensor[t];
    out->inertial_tensor_weighted[t] = s.InertialTensorWeighted[t];
  }
  return 0;
}

// Subhaloes as MergeSubhalos finds them (lists bound first, nests glued):
// hbtu::DetectTrapsGPU at snapshot 7, then SinkTrackId, SnapshotIndexOfSink
// and the IsMerged flags back.
extern "C" int shim_detect_traps(hbtu_handle *h, int64_t nsub, const int64_t *list_off,
                                 const int64_t *id, const float *pos, const float *vel,
                                 const float *mass, const int64_t *nbound, const float *mb_pos,
                                 const float *mb_vel, const int64_t *nest_off,
                                 const int64_t *nest_idx, const int64_t *sink_in,
                                 int64_t *sink_out, int32_t *sink_snap_out, int32_t *merged_out)
{
  std::vector<mock::Subhalo_t> subs(nsub);
  for (int64_t s = 0; s < nsub; s++) {
    mock::Subhalo_t &sub = subs[s];
    for (int64_t i = list_off[s]; i < list_off[s + 1]; i++) {
      mock::Particle_t q;
      q.Id = id[i];
      for (int j = 0; j < 3; j++) {
        q.ComovingPosition[j] = pos[3 * i + j];
        q.PhysicalVelocity[j] = vel[3 * i + j];
      }
      q.Mass = mass[i];
      q.Type = 1;
      sub.Particles.push_back(q);
    }
    sub.Nbound = nbound[s];
    for (int j = 0; j < 3; j++) {
      sub.ComovingMostBoundPosition[j] = mb_pos[3 * s + j];
      sub.PhysicalMostBoundVelocity[j] = mb_vel[3 * s + j];
    }
    for (int64_t k = nest_off[s]; k < nest_off[s + 1]; k++) sub.NestedSubhalos.push_back(nest_idx[k]);
    sub.SinkTrackId = sink_in[s];
    sub.SnapshotIndexOfSink = -1;
  }
  mock::Snapshot_t epoch;
  std::vector<char> merged;
  const hbtu_status rc = hbtu::DetectTrapsGPU(h, subs, epoch, merged);
  if (rc != HBTU_OK) return rc;
  for (int64_t s = 0; s < nsub; s++) {
    sink_out[s] = subs[s].SinkTrackId;
    sink_snap_out[s] = subs[s].SnapshotIndexOfSink;
    merged_out[s] = merged[s];
  }
  return 0;
}

// A forest through hbtu::RecursiveUnbindGPU from `roots` and
// hbtu::TruncateSource on every subhalo (mode 0), or a SubhaloSnapshot_t with
// its member table through hbtu::RefineParticlesGPU (mode 1: haloes'
// members group_off/group_idx, central first; heads heads_off/heads_idx;
// field subhaloes field[0..nfield)).  Out: every subhalo's final list as input
// rows (out_off: nsub+1 offsets) and Nbound.
extern "C" int shim_recursive_unbind(
    hbtu_handle *h, const hbtu_params *par, int32_t mode, int64_t nsub, const int64_t *list_off,
    const int64_t *id, const float *pos, const float *vel, const float *mass, const int32_t *type,
    const int64_t *nbound_prev, const float *ref_pos, const float *ref_vel, const float *mb_pos,
    const float *mb_vel, const int64_t *nest_off, const int64_t *nest_idx, int64_t nroots,
    const int64_t *roots, int64_t nhalo, const int64_t *group_off, const int64_t *group_idx,
    const int64_t *heads_off, const int64_t *heads_idx, int64_t nfield, const int64_t *field,
    float relax, int64_t out_cap, int64_t *out_off, int64_t *out_row, int64_t *out_nbound)
{
  mock::SubhaloSnapshot_t snap;
  snap.index = 7;
  build_subhaloes(snap.Subhalos, nsub, list_off, id, pos, vel, mass, type, nbound_prev, ref_pos,
                  ref_vel, mb_pos, mb_vel, nest_off, nest_idx);
  hbtu_status rc;
  if (mode == 0) {
    rc = hbtu::RecursiveUnbindGPU(h, *par, snap.Subhalos, std::vector<int64_t>(roots, roots + nroots),
                                  snap);
    if (rc == HBTU_OK || rc == HBTU_ERR_NOT_CONVERGED)
      for (auto &s : snap.Subhalos) hbtu::TruncateSource(s, relax);
  } else {
    snap.MemberTable.SubGroups.g.assign(1, std::vector<long>(field, field + nfield));
    for (auto &g : lists_of(nhalo, group_off, group_idx)) snap.MemberTable.SubGroups.g.push_back(g);
    snap.MemberTable.SubGroupsOfHeads = lists_of(nhalo, heads_off, heads_idx);
    for (int64_t s = 0; s < nsub; s++) snap.MemberTable.AllMembers.push_back(s);
    rc = hbtu::RefineParticlesGPU(h, *par, snap, relax);
  }
  if (rc != HBTU_OK && rc != HBTU_ERR_NOT_CONVERGED) return rc;
  int64_t k = 0;
  out_off[0] = 0;
  for (int64_t s = 0; s < nsub; s++) {
    const auto &sub = snap.Subhalos[s];
    for (const auto &p : sub.Particles) {
      if (k >= out_cap) return -1;
      out_row[k++] = p.Row;
    }
    out_off[s + 1] = k;
    out_nbound[s] = sub.Nbound;
  }
  return rc;
}

// SubhaloSnapshot_t::MergeSubhalos through hbtu::MergeSubhalosGPU at snapshot
// `isnap`: subhaloes after their unbinding (lists bound first), nests, the
// haloes' members and heads, SinkTrackId and SnapshotIndexOfDeath.  Out: every
// list as particle Ids with the energies of the re-unbound subhaloes (NaN
// elsewhere), Nbound, SinkTrackId, SnapshotIndexOfSink, SnapshotIndexOfDeath.
extern "C" int shim_merge_subhalos(
    hbtu_handle *h, const hbtu_params *par, int64_t nsub, const int64_t *list_off,
    const int64_t *id, const float *pos, const float *vel, const float *mass, const int32_t *type,
    const int64_t *nbound, const float *ref_pos, const float *ref_vel, const float *mb_pos,
    const float *mb_vel, const int64_t *nest_off, const int64_t *nest_idx, int64_t nhalo,
    const int64_t *group_off, const int64_t *group_idx, const int64_t *heads_off,
    const int64_t *heads_idx, const int64_t *sink, const int32_t *death, int32_t isnap,
    float relax, int64_t out_cap, int64_t *out_off, int64_t *out_id, float *out_energy,
    int64_t *out_nbound, int64_t *out_sink, int32_t *out_sink_snap, int32_t *out_death)
{
  mock::SubhaloSnapshot_t snap;
  snap.index = isnap;
  build_subhaloes(snap.Subhalos, nsub, list_off, id, pos, vel, mass, type, nbound, ref_pos,
                  ref_vel, mb_pos, mb_vel, nest_off, nest_idx);
  for (int64_t s = 0; s < nsub; s++) {
    snap.Subhalos[s].SinkTrackId = sink[s];
    snap.Subhalos[s].SnapshotIndexOfDeath = death[s];
    snap.Subhalos[s].CountParticles();
  }
  snap.MemberTable.SubGroups.g.assign(1, std::vector<long>());
  for (auto &g : lists_of(nhalo, group_off, group_idx)) snap.MemberTable.SubGroups.g.push_back(g);
  snap.MemberTable.SubGroupsOfHeads = lists_of(nhalo, heads_off, heads_idx);
  for (int64_t s = 0; s < nsub; s++) snap.MemberTable.AllMembers.push_back(s);
  std::vector<std::vector<float>> energies;
  const hbtu_status rc = hbtu::MergeSubhalosGPU(h, *par, snap, relax, &energies);
  if (rc != HBTU_OK && rc != HBTU_ERR_NOT_CONVERGED) return rc;
  int64_t k = 0;
  out_off[0] = 0;
  for (int64_t s = 0; s < nsub; s++) {
    const auto &sub = snap.Subhalos[s];
    for (size_t i = 0; i < sub.Particles.size(); i++) {
      if (k >= out_cap) return -1;
      out_id[k] = sub.Particles[i].Id;
      out_energy[k++] = i < energies[s].size() ? energies[s][i] : NAN;
    }
    out_off[s + 1] = k;
    out_nbound[s] = sub.Nbound;
    out_sink[s] = sub.SinkTrackId;
    out_sink_snap[s] = sub.SnapshotIndexOfSink;
    out_death[s] = sub.SnapshotIndexOfDeath;
  }
  return rc;
}
