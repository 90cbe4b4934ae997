// hbtu_subhalo.hpp -- header-only C++ drop-in for HBT+'s unbinding step.
//
//   hbtu::UnbindGPU(handle, params, subhalo, snapshot)
//       replaces  subhalo.Unbind(snapshot)            (src/subhalo_unbind.cpp:263-431)
//   hbtu::UnbindBatchGPU(handle, params, subhaloes, ids, snapshot)
//       replaces  the per-subhalo Unbind loops of SubhaloSnapshot_t::RefineParticles
//                 (src/subhalo_unbind.cpp:471-513), one call per nesting level
//   hbtu::PropertiesGPU(handle, subhaloes, ids, snapshot)
//       replaces  the CalculateProfileProperties + CalculateShape loop at the end
//                 of SubhaloSnapshot_t::UpdateTracks (src/subhalo_tracking.cpp:901-906)
//   hbtu::DetectTrapsGPU(handle, subhaloes, snapshot, merged)
//       replaces  FillHelpers + DetectTraps of SubhaloSnapshot_t::MergeSubhalos
//                 (src/subhalo_merge.cpp:30-180, :193-199)
//
// Templated on the caller's Subhalo_t / Snapshot_t, using the member names of
// src/subhalo.h:24-146 and src/snapshot.h:51-111, so it compiles against the
// reference's own types.  It performs the host-side parts of Unbind:
//   - the sampling shuffle, by the same random_shuffle call (:302);
//   - marshalling Particle_t (AoS) to the C ABI's arrays and back;
//   - applying the permutation of Particles (:409-415);
//   - the bookkeeping of SnapshotIndexOfDeath / SnapshotIndexOfSink / SinkTrackId
//     (:269-273, :365-366, :397-403);
//   - Energies when the caller keeps them (SAVE_BINDING_ENERGY).
// The device does everything else.
#pragma once
#include <algorithm>
#include <cstdint>
#include <type_traits>
#include <vector>

#include "hbtu.h"

namespace hbtu {

struct SubhaloArrays {
  std::vector<int64_t> id;
  std::vector<float> pos, vel, mass;
  std::vector<int32_t> type;
};

namespace detail {

template <class ParticleList>
void gather(const ParticleList &P, SubhaloArrays &a)
{
  for (const auto &p : P) {
    a.id.push_back((int64_t)p.Id);
    for (int j = 0; j < 3; j++) {
      a.pos.push_back((float)p.ComovingPosition[j]);
      a.vel.push_back((float)p.PhysicalVelocity[j]);
    }
    a.mass.push_back((float)p.Mass);
    a.type.push_back((int32_t)p.Type);
  }
}

template <class SubhaloT>
hbtu_state state_of(const SubhaloT &s, int64_t mostbound_id)
{
  hbtu_state st;
  for (int j = 0; j < 3; j++) {
    st.ref_pos[j] = (float)s.ComovingAveragePosition[j];
    st.ref_vel[j] = (float)s.PhysicalAverageVelocity[j];
    st.mostbound_pos[j] = (float)s.ComovingMostBoundPosition[j];
    st.mostbound_vel[j] = (float)s.PhysicalMostBoundVelocity[j];
  }
  st.mostbound_id = mostbound_id;
  return st;
}

// Writes one result back into the subhalo, as Unbind leaves it.
template <class SubhaloT, class SnapshotT>
void apply(SubhaloT &s, const SnapshotT &epoch, const hbtu_result &r, const int64_t *order,
           const float *energy, std::vector<float> *energies)
{
  const int64_t n = (int64_t)s.Particles.size();
  if (r.too_few && s.IsAlive()) s.SnapshotIndexOfDeath = epoch.GetSnapshotIndex();  // :269-273
  if (n >= 2) {
    typename std::decay<decltype(s.Particles)>::type p(n);
    for (int64_t i = 0; i < n; i++) p[i] = s.Particles[order[i]];  // :409-415 / :367-374
    s.Particles.swap(p);
    for (int j = 0; j < 3; j++) {
      s.ComovingAveragePosition[j] = r.ref_pos[j];
      s.PhysicalAverageVelocity[j] = r.ref_vel[j];
      s.ComovingMostBoundPosition[j] = r.mostbound_pos[j];
      s.PhysicalMostBoundVelocity[j] = r.mostbound_vel[j];
      s.SpecificAngularMomentum[j] = r.specific_angmom[j];
    }
    s.SpecificSelfPotentialEnergy = r.specific_potential;
    s.SpecificSelfKineticEnergy = r.specific_kinetic;
    if (r.disrupted && s.IsAlive()) s.SnapshotIndexOfDeath = epoch.GetSnapshotIndex();  // :365-366
    if (r.converged) {                                                                   // :397-403
      if (!s.IsAlive()) s.SnapshotIndexOfDeath = -1;
      if (s.IsTrapped()) {
        s.SnapshotIndexOfSink = -1;
        s.SinkTrackId = -1;
      }
    }
  }
  s.Nbound = r.nbound;
  s.Mbound = r.mbound;
  for (int t = 0; t < 6; t++) {
    s.NboundType[t] = r.nbound_type[t];
    s.MboundType[t] = r.mbound_type[t];
  }
  if (energies) energies->assign(energy, energy + std::min<int64_t>(r.nbound, n));
}

}  // namespace detail

// Subhalo_t::Unbind on the GPU.  `params` is the handle's parameter set.  When
// sampling applies, Particles is shuffled first with the same library call as
// the reference, consuming the same rand() stream.  `energies`: optional
// Subhalo_t::Energies.
template <class SubhaloT, class SnapshotT>
hbtu_status UnbindGPU(hbtu_handle *h, const hbtu_params &params, SubhaloT &sub,
                      const SnapshotT &epoch, std::vector<float> *energies = nullptr)
{
  const int64_t n = (int64_t)sub.Particles.size();
  const int64_t mb_id = n ? (int64_t)sub.Particles[0].Id : -1;
  if (params.max_sample_size > 0 && n > params.max_sample_size)
    std::random_shuffle(sub.Particles.begin(), sub.Particles.end());  // :302
  SubhaloArrays a;
  detail::gather(sub.Particles, a);
  hbtu_particles p{a.id.data(), a.pos.data(), a.vel.data(), a.mass.data(), a.type.data(),
                   HBTU_HOST, 0};
  const hbtu_state st = detail::state_of(sub, mb_id);
  std::vector<int64_t> order(n > 0 ? n : 1);
  std::vector<float> energy(n > 0 ? n : 1);
  hbtu_result r;
  const hbtu_status rc = hbtu_unbind(h, &p, n, &st, order.data(), energy.data(), &r);
  if (rc != HBTU_OK && rc != HBTU_ERR_NOT_CONVERGED) return rc;
  // a pass cap (params.max_passes) that ends the loop early still leaves the
  // subhalo as the last pass left it, as the batch form does
  detail::apply(sub, epoch, r, order.data(), energy.data(), energies);
  return rc;
}

// The independent Unbind calls of one nesting level in one device call:
// subhaloes[ids[k]] for every k (the field and new-born loops of
// RefineParticles, src/subhalo_unbind.cpp:495-510).
template <class SubhaloListT, class SnapshotT>
hbtu_status UnbindBatchGPU(hbtu_handle *h, const hbtu_params &params, SubhaloListT &subhaloes,
                           const std::vector<int64_t> &ids, const SnapshotT &epoch)
{
  SubhaloArrays a;
  std::vector<int64_t> off(1, 0);
  std::vector<hbtu_state> st;
  for (int64_t k : ids) {
    auto &s = subhaloes[k];
    const int64_t n = (int64_t)s.Particles.size();
    const int64_t mb_id = n ? (int64_t)s.Particles[0].Id : -1;
    if (params.max_sample_size > 0 && n > params.max_sample_size)
      std::random_shuffle(s.Particles.begin(), s.Particles.end());
    detail::gather(s.Particles, a);
    off.push_back(off.back() + n);
    st.push_back(detail::state_of(s, mb_id));
  }
  const int64_t nsub = (int64_t)ids.size(), ntot = off.back();
  hbtu_particles p{a.id.data(), a.pos.data(), a.vel.data(), a.mass.data(), a.type.data(),
                   HBTU_HOST, 0};
  std::vector<int64_t> order(ntot > 0 ? ntot : 1);
  std::vector<float> energy(ntot > 0 ? ntot : 1);
  std::vector<hbtu_result> r(nsub > 0 ? nsub : 1);
  const hbtu_status rc =
      hbtu_unbind_batch(h, &p, nsub, off.data(), st.data(), order.data(), energy.data(), r.data());
  if (rc != HBTU_OK && rc != HBTU_ERR_NOT_CONVERGED) return rc;
  for (int64_t k = 0; k < nsub; k++)
    detail::apply(subhaloes[ids[k]], epoch, r[k], order.data() + off[k], energy.data() + off[k],
                  (std::vector<float> *)nullptr);
  return rc;
}

// Subhalo_t::CalculateProfileProperties and ::CalculateShape
// (src/subhalo.cpp:242-398) of subhaloes[ids[k]] for every k, in one device
// call, on their bound particles (Particles[0 .. Nbound), most-bound first, as
// Unbind leaves them).  A subhalo with Nbound <= 1 is left as it is, as in the
// reference.
template <class SubhaloListT, class SnapshotT>
hbtu_status PropertiesGPU(hbtu_handle *h, SubhaloListT &subhaloes, const std::vector<int64_t> &ids,
                          const SnapshotT &epoch)
{
  SubhaloArrays a;
  std::vector<int64_t> off(1, 0), order;
  std::vector<hbtu_result> r;
  std::vector<float> last_max;
  std::vector<int32_t> last_snap;
  for (int64_t k : ids) {
    auto &s = subhaloes[k];
    const int64_t n = (int64_t)s.Particles.size();
    detail::gather(s.Particles, a);
    for (int64_t i = 0; i < n; i++) order.push_back(i);  // Particles are in bound order already
    off.push_back(off.back() + n);
    hbtu_result q{};
    q.nbound = (int64_t)s.Nbound;
    q.mbound = (float)s.Mbound;
    for (int j = 0; j < 3; j++) q.mostbound_pos[j] = (float)s.ComovingMostBoundPosition[j];
    r.push_back(q);
    last_max.push_back((float)s.LastMaxVmaxPhysical);
    last_snap.push_back((int32_t)s.SnapshotIndexOfLastMaxVmax);
  }
  const int64_t nsub = (int64_t)ids.size();
  if (nsub == 0) return HBTU_OK;
  hbtu_particles p{a.id.data(), a.pos.data(), a.vel.data(), a.mass.data(), a.type.data(),
                   HBTU_HOST, 0};
  if (order.empty()) order.push_back(0);
  std::vector<hbtu_props> out(nsub);
  const hbtu_status rc =
      hbtu_subhalo_properties(h, &p, nsub, off.data(), order.data(), r.data(), last_max.data(),
                              last_snap.data(), (int32_t)epoch.GetSnapshotIndex(), out.data());
  if (rc != HBTU_OK) return rc;
  for (int64_t k = 0; k < nsub; k++) {
    auto &s = subhaloes[ids[k]];
    if (s.Nbound <= 1) continue;  // subhalo.cpp:264-282, :339-351
    const hbtu_props &q = out[k];
    s.RmaxComoving = q.rmax_comoving;
    s.VmaxPhysical = q.vmax_physical;
    s.LastMaxVmaxPhysical = q.last_max_vmax_physical;
    s.SnapshotIndexOfLastMaxVmax = q.snapshot_of_last_max_vmax;
    s.R2SigmaComoving = q.r2sigma_comoving;
    s.RHalfComoving = q.rhalf_comoving;
    s.BoundR200CritComoving = q.r200crit_comoving;
    s.BoundM200Crit = q.m200crit;
    for (int t = 0; t < 6; t++) {
      s.InertialTensor[t] = q.inertial_tensor[t];
      s.InertialTensorWeighted[t] = q.inertial_tensor_weighted[t];
    }
  }
  return HBTU_OK;
}

// FillHelpers + DetectTraps of SubhaloSnapshot_t::MergeSubhalos
// (src/subhalo_merge.cpp:30-180) for every subhalo, on the GPU.  Call it where
// MergeSubhalos fills its helpers, with the head nests glued (GlueHeadNests):
// the host of a subhalo is the subhalo whose NestedSubhalos lists it (the last
// one in index order).  Writes SinkTrackId and SnapshotIndexOfSink of the
// subhaloes trapped now and returns, per subhalo, the IsMerged flag of its
// helper (it swallows a subhalo with Nbound > 1).  The core of a subhalo reads
// its first min(Nbound, 20) particles, so only those are sent.
template <class SubhaloListT, class SnapshotT>
hbtu_status DetectTrapsGPU(hbtu_handle *h, SubhaloListT &subhaloes, const SnapshotT &epoch,
                           std::vector<char> &merged)
{
  const int64_t nsub = (int64_t)subhaloes.size();
  merged.assign(nsub, 0);
  if (nsub == 0) return HBTU_OK;
  SubhaloArrays a;
  std::vector<int64_t> off(1, 0), nbound(nsub), host(nsub, -1), sink(nsub);
  std::vector<float> mbp(3 * nsub), mbv(3 * nsub);
  std::vector<int32_t> sink_snap(nsub), flag(nsub);
  for (int64_t i = 0; i < nsub; i++) {
    auto &s = subhaloes[i];
    for (auto c : s.NestedSubhalos) host[(int64_t)c] = i;  // FillHostTrackIds (:162-171)
    const int64_t nb = (int64_t)s.Nbound;
    const int64_t ncore = std::min<int64_t>({nb > 0 ? nb : 0, (int64_t)s.Particles.size(), 20});
    typename std::decay<decltype(s.Particles)>::type core(s.Particles.begin(),
                                                          s.Particles.begin() + ncore);
    detail::gather(core, a);
    off.push_back(off.back() + ncore);
    nbound[i] = nb;
    sink[i] = (int64_t)s.SinkTrackId;
    sink_snap[i] = (int32_t)s.SnapshotIndexOfSink;
    for (int j = 0; j < 3; j++) {
      mbp[3 * i + j] = (float)s.ComovingMostBoundPosition[j];
      mbv[3 * i + j] = (float)s.PhysicalMostBoundVelocity[j];
    }
  }
  if (a.mass.empty()) {  // no particles at all: keep the pointers valid
    a.id.push_back(0);
    a.mass.push_back(0.f);
    a.type.push_back(1);
    for (int j = 0; j < 3; j++) {
      a.pos.push_back(0.f);
      a.vel.push_back(0.f);
    }
  }
  hbtu_particles p{a.id.data(), a.pos.data(), a.vel.data(), a.mass.data(), a.type.data(),
                   HBTU_HOST, 0};
  const hbtu_status rc = hbtu_merge_detect(h, &p, nsub, off.data(), nbound.data(), host.data(),
                                           mbp.data(), mbv.data(),
                                           (int32_t)epoch.GetSnapshotIndex(), sink.data(),
                                           sink_snap.data(), flag.data(), nullptr);
  if (rc != HBTU_OK) return rc;
  for (int64_t i = 0; i < nsub; i++) {
    auto &s = subhaloes[i];
    s.SinkTrackId = sink[i];
    s.SnapshotIndexOfSink = sink_snap[i];
    merged[i] = flag[i] != 0;
  }
  return HBTU_OK;
}

}  // namespace hbtu
