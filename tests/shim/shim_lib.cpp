// shim_lib.cpp -- test harness of include/hbtu_subhalo.hpp.
//
// Stand-ins for HBT+'s Particle_t / Subhalo_t / Snapshot_t with the member
// names and types of src/snapshot.h:51-72 and src/subhalo.h:24-146 (HBT_INT8,
// float HBTReal), so the shim is exercised exactly as the reference would use
// it.  shim_unbind() builds one subhalo, calls hbtu::UnbindGPU and reports the
// subhalo as Unbind leaves it.
#include <array>
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
};
struct Snapshot_t {
  int GetSnapshotIndex() const { return 7; }
};
}  // namespace mock

extern "C" int shim_unbind(hbtu_handle *h, const hbtu_params *par, int64_t n, const int64_t *id,
                           const float *pos, const float *vel, const float *mass,
                           const int32_t *type, const hbtu_state *st, int64_t *out_id,
                           float *out_energy, hbtu_result *out, int32_t *death)
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
  const hbtu_status rc = hbtu::UnbindGPU(h, *par, s, epoch, &energies);
  if (rc != HBTU_OK) return rc;
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
  return HBTU_OK;
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
