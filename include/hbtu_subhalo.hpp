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
//   hbtu::RecursiveUnbindGPU(handle, params, subhaloes, roots, snapshot)
//       replaces  Subhalo_t::RecursiveUnbind from each root (src/subhalo_unbind.cpp:432-447),
//                 one device call per nesting depth, deepest first
//   hbtu::TruncateSource(subhalo, relax)
//       replaces  Subhalo_t::TruncateSource (src/subhalo_unbind.cpp:449-458)
//   hbtu::RefineParticlesGPU(handle, params, subhalo_snapshot, relax)
//       replaces  SubhaloSnapshot_t::RefineParticles (src/subhalo_unbind.cpp:460-516)
//   hbtu::MergeSubhalosGPU(handle, params, subhalo_snapshot, relax)
//       replaces  SubhaloSnapshot_t::MergeSubhalos with MergeTrappedSubhalos on
//                 (src/subhalo_merge.cpp:187-262)
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
#include <unordered_set>
#include <utility>
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
// `energies` (optional): Subhalo_t::Energies of each subhalo of the call, in
// the order of `ids`.
template <class SubhaloListT, class SnapshotT>
hbtu_status UnbindBatchGPU(hbtu_handle *h, const hbtu_params &params, SubhaloListT &subhaloes,
                           const std::vector<int64_t> &ids, const SnapshotT &epoch,
                           std::vector<std::vector<float>> *energies = nullptr)
{
  if (energies) energies->assign(ids.size(), std::vector<float>());
  if (ids.empty()) return HBTU_OK;
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
                  energies ? &(*energies)[k] : (std::vector<float> *)nullptr);
  return rc;
}

// Subhalo_t::TruncateSource (src/subhalo_unbind.cpp:449-458): Particles cut to
// Nbound * SourceSubRelaxFactor (`relax`), the product formed in float and
// truncated as the reference forms it (HBTInt times HBTReal).
template <class SubhaloT>
void TruncateSource(SubhaloT &s, float relax)
{
  int64_t n = (int64_t)s.Nbound;
  if (n > 1) n = (int64_t)((float)s.Nbound * relax);
  if (n > (int64_t)s.Particles.size()) n = (int64_t)s.Particles.size();
  s.Particles.resize(n);
}

// Subhalo_t::RecursiveUnbind (src/subhalo_unbind.cpp:432-447) from each of
// `roots`, for the whole forest below them: a nested subhalo is unbound before
// its host, and its unbound tail (Particles[Nbound:]) is appended to the host's
// list, in the order of NestedSubhalos, before the host is unbound; an orphan
// (Nbound <= 1 on entry) is unbound on its own particles but keeps the
// extended list to hand on.  The subhaloes of one nesting depth do not depend
// on each other, so each depth is one hbtu_unbind_batch call, deepest first: a
// forest costs one device call per level.  A subhalo listed in two nests is
// unbound once, at its first appearance (depth-first order).
template <class SubhaloListT, class SnapshotT>
hbtu_status RecursiveUnbindGPU(hbtu_handle *h, const hbtu_params &params, SubhaloListT &subhaloes,
                               const std::vector<int64_t> &roots, const SnapshotT &epoch)
{
  const int64_t nsub = (int64_t)subhaloes.size();
  std::vector<int64_t> depth(nsub, -1);
  int64_t maxd = -1;
  std::vector<std::pair<int64_t, int64_t>> stack;
  for (auto it = roots.rbegin(); it != roots.rend(); ++it) stack.emplace_back(*it, 0);
  while (!stack.empty()) {  // depth-first preorder, first appearance wins
    const auto top = stack.back();
    stack.pop_back();
    if (depth[top.first] >= 0) continue;
    depth[top.first] = top.second;
    maxd = std::max(maxd, top.second);
    const auto &nest = subhaloes[top.first].NestedSubhalos;
    for (auto it = nest.rbegin(); it != nest.rend(); ++it)
      stack.emplace_back((int64_t)*it, top.second + 1);
  }
  hbtu_status worst = HBTU_OK;
  for (int64_t d = maxd; d >= 0; d--) {
    std::vector<int64_t> level;
    for (int64_t s = 0; s < nsub; s++)
      if (depth[s] == d) level.push_back(s);
    std::vector<typename std::decay<decltype(subhaloes[0].Particles)>::type> extended;
    std::vector<char> orphan(level.size());
    for (size_t k = 0; k < level.size(); k++) {
      auto &sub = subhaloes[level[k]];
      orphan[k] = sub.Nbound <= 1;
      auto ext = sub.Particles;
      for (auto c : sub.NestedSubhalos) {
        const auto &child = subhaloes[(int64_t)c];
        if (depth[(int64_t)c] != d + 1) continue;  // unbound at another appearance
        ext.insert(ext.end(), child.Particles.begin() + (int64_t)child.Nbound,
                   child.Particles.end());
      }
      if (orphan[k]) {
        extended.push_back(std::move(ext));  // its own particles are unbound
      } else {
        sub.Particles.swap(ext);
        extended.emplace_back();
      }
    }
    const hbtu_status rc = UnbindBatchGPU(h, params, subhaloes, level, epoch);
    if (rc != HBTU_OK && rc != HBTU_ERR_NOT_CONVERGED) return rc;
    if (rc != HBTU_OK) worst = rc;
    for (size_t k = 0; k < level.size(); k++)
      if (orphan[k]) subhaloes[level[k]].Particles.swap(extended[k]);  // :444-446
  }
  return worst;
}

// SubhaloSnapshot_t::RefineParticles (src/subhalo_unbind.cpp:460-516): each
// halo's other top-level subhaloes join its central's nest, the forests of all
// haloes go through RecursiveUnbindGPU together (one device call per depth),
// the field and new-born subhaloes through one UnbindBatchGPU call, and every
// list is cut by TruncateSource.  `relax` is SourceSubRelaxFactor.
template <class SubhaloSnapshotT>
hbtu_status RefineParticlesGPU(hbtu_handle *h, const hbtu_params &params, SubhaloSnapshotT &snap,
                               float relax)
{
  auto &subs = snap.Subhalos;
  auto &table = snap.MemberTable;
  const int64_t nhalo = (int64_t)table.SubGroups.size();
  std::vector<int64_t> roots, nest_size(nhalo, -1);
  for (int64_t g = 0; g < nhalo; g++) {  // :481-494
    const auto &group = table.SubGroups[g];
    if (group.size() == 0) continue;
    auto &nests = subs[(int64_t)group[0]].NestedSubhalos;
    nest_size[g] = (int64_t)nests.size();
    const auto &heads = table.SubGroupsOfHeads[g];
    if (heads.size() > 1) nests.insert(nests.end(), heads.begin() + 1, heads.end());
    roots.push_back((int64_t)group[0]);
  }
  const hbtu_status rc = RecursiveUnbindGPU(h, params, subs, roots, snap);
  for (int64_t g = 0; g < nhalo; g++)  // restore the nests, also after an error
    if (nest_size[g] >= 0) subs[(int64_t)table.SubGroups[g][0]].NestedSubhalos.resize(nest_size[g]);
  if (rc != HBTU_OK && rc != HBTU_ERR_NOT_CONVERGED) return rc;
  std::vector<int64_t> plain;  // field subhaloes, then new-born ones (:497-510)
  const auto &field = table.SubGroups[-1];
  for (int64_t i = 0; i < (int64_t)field.size(); i++) plain.push_back((int64_t)field[i]);
  for (int64_t i = (int64_t)table.AllMembers.size(); i < (int64_t)subs.size(); i++)
    plain.push_back(i);
  const hbtu_status rc2 = UnbindBatchGPU(h, params, subs, plain, snap);
  if (rc2 != HBTU_OK && rc2 != HBTU_ERR_NOT_CONVERGED) return rc2;
  for (auto &s : subs) TruncateSource(s, relax);  // :511-512
  return rc != HBTU_OK ? rc : rc2;
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


namespace detail {

// Subhalo_t::MergeTo (src/subhalo_merge.cpp:244-262): the sink receives the
// particles whose Ids it does not hold yet, in the subhalo's order, and the
// subhalo's Nbound; the subhalo keeps its most-bound particle.
template <class SubhaloT>
void merge_to(SubhaloT &sat, SubhaloT &host)
{
  if (sat.Nbound <= 1) return;  // orphans and nulls
  std::unordered_set<int64_t> ids(host.Particles.size() + sat.Particles.size());
  for (const auto &p : host.Particles) ids.insert((int64_t)p.Id);
  host.Particles.reserve(host.Particles.size() + sat.Particles.size());
  for (const auto &p : sat.Particles)
    if (ids.insert((int64_t)p.Id).second) host.Particles.push_back(p);
  host.Nbound += sat.Nbound;
  sat.Particles.resize(1);
  sat.Nbound = 1;
  sat.CountParticles();
}

// SubhaloSnapshot_t::MergeRecursive (:222-232): depth first, nested subhaloes
// before their host; a trapped subhalo that is alive merges into its sink.
template <class SubhaloListT>
void merge_recursive(SubhaloListT &subs, int64_t root, int snapshot_index)
{
  std::vector<std::pair<int64_t, bool>> stack(1, std::make_pair(root, false));
  while (!stack.empty()) {
    const auto top = stack.back();
    stack.pop_back();
    auto &sat = subs[top.first];
    if (!top.second) {
      stack.emplace_back(top.first, true);
      const auto &nest = sat.NestedSubhalos;
      for (auto it = nest.rbegin(); it != nest.rend(); ++it)
        stack.emplace_back((int64_t)*it, false);
      continue;
    }
    if (sat.IsTrapped() && sat.IsAlive()) {
      merge_to(sat, subs[(int64_t)sat.SinkTrackId]);
      sat.SnapshotIndexOfDeath = snapshot_index;
    }
  }
}

}  // namespace detail

// SubhaloSnapshot_t::MergeSubhalos with MergeTrappedSubhalos on
// (src/subhalo_merge.cpp:187-220): the heads of each halo join its central's
// nest (GlueHeadNests), DetectTrapsGPU finds the sinks on the device, trapped
// subhaloes merge into their sinks depth first on the host, every subhalo that
// swallowed one with Nbound > 1 is unbound again in one UnbindBatchGPU call and
// cut by TruncateSource, and the nests are restored (UnglueHeadNests).
// `energies` (optional): Subhalo_t::Energies of the re-unbound subhaloes
// (empty for the others).
template <class SubhaloSnapshotT>
hbtu_status MergeSubhalosGPU(hbtu_handle *h, const hbtu_params &params, SubhaloSnapshotT &snap,
                             float relax, std::vector<std::vector<float>> *energies = nullptr)
{
  auto &subs = snap.Subhalos;
  auto &table = snap.MemberTable;
  const int64_t nhalo = (int64_t)table.SubGroups.size();
  std::vector<int64_t> nest_size(nhalo, -1);
  for (int64_t g = 0; g < nhalo; g++) {  // GlueHeadNests (src/subhalo_tracking.cpp:843-862)
    const auto &group = table.SubGroups[g];
    if (group.size() == 0) continue;
    auto &nests = subs[(int64_t)group[0]].NestedSubhalos;
    nest_size[g] = (int64_t)nests.size();
    const auto &heads = table.SubGroupsOfHeads[g];
    if (heads.size() > 1) nests.insert(nests.end(), heads.begin() + 1, heads.end());
  }
  std::vector<char> merged;
  hbtu_status rc = DetectTrapsGPU(h, subs, snap, merged);
  std::vector<int64_t> again;
  if (rc == HBTU_OK) {
    const int isnap = (int)snap.GetSnapshotIndex();
    for (int64_t g = 0; g < nhalo; g++)
      if (table.SubGroups[g].size())
        detail::merge_recursive(subs, (int64_t)table.SubGroups[g][0], isnap);
    for (int64_t s = 0; s < (int64_t)subs.size(); s++)
      if (merged[s]) again.push_back(s);
  }
  for (int64_t g = 0; g < nhalo; g++)  // UnglueHeadNests (:863-874)
    if (nest_size[g] >= 0) subs[(int64_t)table.SubGroups[g][0]].NestedSubhalos.resize(nest_size[g]);
  if (rc != HBTU_OK) return rc;
  std::vector<std::vector<float>> en;
  rc = UnbindBatchGPU(h, params, subs, again, snap, energies ? &en : nullptr);
  if (rc != HBTU_OK && rc != HBTU_ERR_NOT_CONVERGED) return rc;
  for (int64_t s : again) TruncateSource(subs[s], relax);
  if (energies) {
    energies->assign(subs.size(), std::vector<float>());
    for (size_t k = 0; k < again.size(); k++) (*energies)[again[k]].swap(en[k]);
  }
  return rc;
}

}  // namespace hbtu
