/* hbt_oracle.c -- CPU oracle (plain C + OpenMP) for the HBT+ unbinding path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU implementation and the
 * timed CPU baseline.  The product (hbtplus_gb300/) never links this file.
 *
 * Every function restates one piece of the reference and cites it.  The float
 * (HBTReal) versus double arithmetic of the reference is kept operation by
 * operation, because the bound set is decided by the sign of a float energy:
 *   - HBTReal members and products of two HBTReals are float,
 *   - the tree walk, node moments and frame sums are double,
 *   - results are rounded to float where the reference stores them.
 * Build with -ffp-contract=off so no multiply-add is fused.
 */
#define _DEFAULT_SOURCE 1
#include "hbt_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Parameters as the reference stores them (src/config_parser.cpp:95-103).  */
typedef struct {
  float eps, theta2, box, boxhalf, res, reshalf, G, Hz, a, prec;
  int periodic, refine;
  int64_t minpart, maxsample;
} dpar;

static void derive(const hbto_params *p, dpar *d)
{
  float th = (float)p->open_angle;
  d->eps = (float)p->softening;
  d->theta2 = th * th;                       /* TreeNodeOpenAngleSquare, :103 */
  d->box = (float)p->box_size;
  d->boxhalf = (float)((double)d->box / 2.); /* BoxHalf, :100 */
  d->res = (float)((double)d->eps * 0.1);    /* TreeNodeResolution, :101 */
  d->reshalf = (float)((double)d->res / 2.); /* TreeNodeResolutionHalf, :102 */
  d->G = (float)p->G;
  d->Hz = (float)p->hubble;
  d->a = (float)p->scale_factor;
  d->prec = (float)p->bound_mass_precision;
  d->periodic = p->periodic != 0;
  d->minpart = p->min_num_part;
  d->maxsample = p->max_sample_size;
  /* RefineMostboundParticle only acts with sampling (subhalo_unbind.cpp:266) */
  d->refine = (p->max_sample_size > 0 && p->refine_mostbound);
}

/* NEAREST (src/config_parser.h:142) on a double and on a float operand. */
static inline double nearest_d(double x, const dpar *d)
{
  return x > d->boxhalf ? x - d->box : (x < -d->boxhalf ? x + d->box : x);
}
static inline float nearest_f(float x, const dpar *d)
{
  return x > d->boxhalf ? x - d->box : (x < -d->boxhalf ? x + d->box : x);
}

/* Snapshot_t::RelativeVelocity, src/snapshot.h:100-111 (float arithmetic). */
static inline void relvel(const float *tp, const float *tv, const float *rp, const float *rv,
                          float *dv, const dpar *d)
{
  for (int j = 0; j < 3; j++) {
    float dx = tp[j] - rp[j];
    if (d->periodic) dx = nearest_f(dx, d);
    dv[j] = tv[j] - rv[j];
    dv[j] += d->Hz * d->a * dx;
  }
}

/* ------------------------------------------------------------------------ */
/* Octree: OctTree_t<TreeCell_t<float>> + GravityTree_t.
 * Node ids [0,np) are tree particles (view positions), ids >= np are cells
 * (src/oct_tree.h:51, tpp:9-14).  The root is np.                            */
typedef struct {
  /* view of the particles in the tree (EnergySnapshot_t, subhalo_unbind.cpp:68-107) */
  const int64_t *pid;
  const float *pos, *mass;
  float mass_factor;
  int64_t np;
  /* cells */
  int64_t ncell, capcell;
  int64_t (*sons)[8];
  float (*s)[3];
  float *len, *cmass;
  int64_t *sibling, *nextnode;
  int64_t *next_from_particle;
  int64_t cap_np;
} otree;

static void tree_init(otree *t)
{
  memset(t, 0, sizeof(*t));
}

static void tree_free(otree *t)
{
  free(t->sons);
  free(t->s);
  free(t->len);
  free(t->cmass);
  free(t->sibling);
  free(t->nextnode);
  free(t->next_from_particle);
  tree_init(t);
}

static inline const float *tpos(const otree *t, int64_t i) { return t->pos + 3 * t->pid[i]; }
/* EnergySnapshot_t::GetMass: Mass*MassFactor in float (subhalo_unbind.cpp:96-99) */
static inline float tmass(const otree *t, int64_t i) { return t->mass[t->pid[i]] * t->mass_factor; }

static int64_t append_cell(otree *t) /* OctTree_t::AppendCell, tpp:9-14 */
{
  if (t->ncell == t->capcell) {
    int64_t c = t->capcell ? 2 * t->capcell : 64;
    t->sons = realloc(t->sons, c * sizeof(*t->sons));
    t->s = realloc(t->s, c * sizeof(*t->s));
    t->len = realloc(t->len, c * sizeof(float));
    t->cmass = realloc(t->cmass, c * sizeof(float));
    t->sibling = realloc(t->sibling, c * sizeof(int64_t));
    t->nextnode = realloc(t->nextnode, c * sizeof(int64_t));
    t->capcell = c;
  }
  for (int k = 0; k < 8; k++) t->sons[t->ncell][k] = -1;
  return t->ncell++;
}

static void update_internal(otree *t, int64_t no, int64_t sib, double len, const dpar *d);

/* GravityTree_t::ProcessNode, src/gravity_tree.cpp:25-46 */
static void process_node(otree *t, int64_t nodeid, int64_t nextid, double *mass, double com[3],
                         double len, const dpar *d)
{
  if (nodeid < t->np) {
    double thismass = tmass(t, nodeid);
    const float *x = tpos(t, nodeid);
    *mass += thismass;
    for (int k = 0; k < 3; k++) com[k] += x[k] * thismass;
    t->next_from_particle[nodeid] = nextid;
  } else {
    if (len >= d->res)
      update_internal(t, nodeid, nextid, len / 2., d);
    else
      update_internal(t, nodeid, nextid, len, d);
    int64_t c = nodeid - t->np;
    double thismass = t->cmass[c];
    *mass += thismass;
    for (int k = 0; k < 3; k++) com[k] += t->s[c][k] * thismass;
  }
}

/* GravityTree_t::UpdateInternalNodes + FillNodeCenter, gravity_tree.cpp:18-23, 48-77 */
static void update_internal(otree *t, int64_t no, int64_t sib, double len, const dpar *d)
{
  int64_t c = no - t->np, sons[8], p, pp;
  int i, jj;
  double mass = 0., com[3] = {0., 0., 0.};
  memcpy(sons, t->sons[c], sizeof(sons));
  t->len[c] = (float)len;
  t->sibling[c] = sib;
  for (i = 0; sons[i] < 0; i++) {
  }
  jj = i;
  pp = sons[jj];
  t->nextnode[c] = pp;
  for (i++; i < 8; i++) {
    if (sons[i] >= 0) {
      p = pp;
      jj = i;
      pp = sons[jj];
      process_node(t, p, pp, &mass, com, len, d);
    }
  }
  process_node(t, pp, sib, &mass, com, len, d);
  t->cmass[c] = (float)mass;
  for (int k = 0; k < 3; k++) t->s[c][k] = (float)(com[k] / mass);
}

/* drand48 draws of the calling thread's current subhalo (one subhalo runs on
 * one thread): reported per subhalo, since a process-global stream shared by
 * threads makes those splits depend on thread timing. */
static _Thread_local int64_t random_splits;

/* OctTree_t::Build, src/oct_tree.tpp:16-144, followed by UpdateInternalNodes. */
static void tree_build(otree *t, const int64_t *pid, int64_t np, const float *pos,
                       const float *mass, float mass_factor, const dpar *d)
{
  double xmin[3], xmax[3], Center[3], center[3], Len, Lenhalf, lenhalf;
  int64_t i, nodeid, subid, sub;
  int j;

  t->pid = pid;
  t->pos = pos;
  t->mass = mass;
  t->mass_factor = mass_factor;
  t->np = np;
  t->ncell = 0;
  if (np > t->cap_np) {
    t->next_from_particle = realloc(t->next_from_particle, np * sizeof(int64_t));
    t->cap_np = np;
  }
  if (np <= 0) return;

  for (j = 0; j < 3; j++) xmin[j] = xmax[j] = tpos(t, 0)[j];
  for (i = 1; i < np; i++)
    for (j = 0; j < 3; j++) {
      const float x = tpos(t, i)[j];
      if (x > xmax[j])
        xmax[j] = x;
      else if (x < xmin[j])
        xmin[j] = x;
    }
  for (j = 1, Len = xmax[0] - xmin[0]; j < 3; j++)
    if ((xmax[j] - xmin[j]) > Len) Len = xmax[j] - xmin[j];
  for (j = 0; j < 3; j++) Center[j] = 0.5 * (xmax[j] + xmin[j]);
  Lenhalf = 0.5 * Len;

  append_cell(t); /* root, id np */

  for (i = 0; i < np; i++) {
    const float *x = tpos(t, i);
    nodeid = np;
    lenhalf = Lenhalf;
    for (j = 0; j < 3; j++) center[j] = Center[j];
    for (;;) {
      lenhalf *= 0.5;
      sub = 0;
      for (j = 0; j < 3; j++) {
        if (x[j] > center[j]) {
          center[j] += lenhalf;
          sub += (1 << j);
        } else {
          center[j] -= lenhalf;
        }
      }
      subid = t->sons[nodeid - np][sub];
      if (subid < 0) {
        t->sons[nodeid - np][sub] = i;
        break;
      } else if (subid < np) {
        int64_t newnodeid = np + t->ncell;
        append_cell(t);
        t->sons[nodeid - np][sub] = newnodeid;
        nodeid = newnodeid;
        if (lenhalf < d->reshalf) {
          /* particles closer than the resolution: random octant (tpp:112-123) */
          random_splits++;
          sub = (int64_t)(8.0 * drand48());
          if (sub >= 8) sub = 7;
        } else {
          const float *y = tpos(t, subid);
          sub = 0;
          if (y[0] > center[0]) sub += 1;
          if (y[1] > center[1]) sub += 2;
          if (y[2] > center[2]) sub += 4;
        }
        t->sons[nodeid - np][sub] = subid;
      } else {
        nodeid = subid;
      }
    }
  }
  update_internal(t, np, -1, Len, d);
}

/* GravityTree_t::EvaluatePotential, src/gravity_tree.cpp:79-164.
 * Returns the specific physical potential; *cnt counts summed contributions. */
static double eval_potential(const otree *t, const float *tp, float targetmass, const dpar *d,
                             int64_t *cnt)
{
  const double px = tp[0], py = tp[1], pz = tp[2];
  const double h = 2.8 * d->eps;
  const double h_inv = 1.0 / h;
  double pot = targetmass / d->eps; /* float division, cancels the self term */
  int64_t no = t->np, n = 0;

  if (t->np <= 0) return 0.;
  while (no >= 0) {
    double dx, dy, dz, mass, r2, r;
    if (no < t->np) {
      const float *x = tpos(t, no);
      dx = x[0] - px;
      dy = x[1] - py;
      dz = x[2] - pz;
      if (d->periodic) {
        dx = nearest_d(dx, d);
        dy = nearest_d(dy, d);
        dz = nearest_d(dz, d);
      }
      mass = tmass(t, no);
      no = t->next_from_particle[no];
      r2 = dx * dx + dy * dy + dz * dz;
    } else {
      int64_t c = no - t->np;
      dx = t->s[c][0] - px;
      dy = t->s[c][1] - py;
      dz = t->s[c][2] - pz;
      if (d->periodic) {
        dx = nearest_d(dx, d);
        dy = nearest_d(dy, d);
        dz = nearest_d(dz, d);
      }
      mass = t->cmass[c];
      r2 = dx * dx + dy * dy + dz * dz;
      {
        const float len2 = t->len[c] * t->len[c]; /* float product */
        if (len2 > r2 * d->theta2) {
          no = t->nextnode[c];
          continue;
        }
      }
      no = t->sibling[c];
    }
    r = sqrt(r2);
    if (r >= h)
      pot -= mass / r;
    else {
      /* cubic-spline softened potential (Springel, Yoshida & White 2001) */
      double u = r * h_inv, wp;
      if (u < 0.5)
        wp = -2.8 + u * u * (5.333333333333 + u * u * (6.4 * u - 9.6));
      else
        wp = -3.2 + 0.066666666667 / u +
             u * u * (10.666666666667 + u * (-16.0 + u * (9.6 - 2.133333333333 * u)));
      pot += mass * h_inv * wp;
    }
    n++;
  }
  if (cnt) *cnt += n;
  return pot * d->G / d->a;
}

/* GravityTree_t::BindingEnergy, src/gravity_tree.cpp:166-175 */
static double binding_energy(const otree *t, const float *x, const float *v, const float *rp,
                             const float *rv, float targetmass, const dpar *d, int64_t *cnt)
{
  double pot = eval_potential(t, x, targetmass, d, cnt);
  float dv[3];
  relvel(x, v, rp, rv, dv, d);
  return (dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]) * 0.5 + pot;
}

/* ------------------------------------------------------------------------ */
/* PartitionBindingEnergy, src/subhalo_unbind.cpp:21-58.                    */
static int64_t partition_energy(float *E, int64_t *pid, int64_t len)
{
  if (len == 0) return 0;
  if (len == 1) return E[0] < 0;
  float tE = E[0];
  int64_t tp = pid[0];
  int64_t f = 0, b = len;
  for (;;) {
    for (;;) {
      b--;
      if (b == f) {
        E[f] = tE;
        pid[f] = tp;
        if (tE < 0) b++;
        return b;
      }
      if (E[b] < 0) break;
    }
    E[f] = E[b];
    pid[f] = pid[b];
    for (;;) {
      f++;
      if (f == b) {
        E[b] = tE;
        pid[b] = tp;
        if (tE < 0) b++;
        return b;
      }
      if (E[f] > 0) break;
    }
    E[b] = E[f];
    pid[b] = pid[f];
  }
}

int64_t hbto_partition(float *E, int64_t *idx, int64_t len) { return partition_energy(E, idx, len); }

/* Ascending sort of (E, pid) records by E (CompEnergy, subhalo_unbind.cpp:17-20).
 * std::sort is not stable; this merge sort is, so equal energies keep their
 * incoming order.  Orders are therefore compared modulo exact-E ties. */
static void sort_energy(float *E, int64_t *pid, int64_t n, float *tE, int64_t *tp)
{
  if (n < 2) return;
  if (n <= 16) {
    for (int64_t i = 1; i < n; i++) {
      float e = E[i];
      int64_t p = pid[i], j = i - 1;
      while (j >= 0 && E[j] > e) {
        E[j + 1] = E[j];
        pid[j + 1] = pid[j];
        j--;
      }
      E[j + 1] = e;
      pid[j + 1] = p;
    }
    return;
  }
  int64_t h = n / 2;
  sort_energy(E, pid, h, tE, tp);
  sort_energy(E + h, pid + h, n - h, tE, tp);
  int64_t i = 0, j = h, k = 0;
  while (i < h && j < n) {
    if (E[j] < E[i]) {
      tE[k] = E[j];
      tp[k++] = pid[j++];
    } else {
      tE[k] = E[i];
      tp[k++] = pid[i++];
    }
  }
  while (i < h) {
    tE[k] = E[i];
    tp[k++] = pid[i++];
  }
  while (j < n) {
    tE[k] = E[j];
    tp[k++] = pid[j++];
  }
  memcpy(E, tE, n * sizeof(float));
  memcpy(pid, tp, n * sizeof(int64_t));
}

static void sort_energy_alloc(float *E, int64_t *pid, int64_t n)
{
  if (n < 2) return;
  float *tE = malloc(n * sizeof(float));
  int64_t *tp = malloc(n * sizeof(int64_t));
  sort_energy(E, pid, n, tE, tp);
  free(tE);
  free(tp);
}

/* ------------------------------------------------------------------------ */
/* EnergySnapshot_t averages over the first num entries of the energy list.  */
typedef struct {
  const float *pos, *vel, *mass;
  const int64_t *pid; /* Elist pids */
  const float *E;
} eview;

/* EnergySnapshot_t::AverageVelocity, subhalo_unbind.cpp:108-138 */
static double average_velocity(const eview *v, int64_t num, float cov[3], int nthr)
{
  double svx = 0., svy = 0., svz = 0., msum = 0.;
  if (num == 0) return 0.;
  if (num == 1) {
    memcpy(cov, v->vel + 3 * v->pid[0], 3 * sizeof(float));
    return v->mass[v->pid[0]];
  }
#pragma omp parallel for reduction(+ : msum, svx, svy, svz) if (num > 100) num_threads(nthr)
  for (int64_t i = 0; i < num; i++) {
    const float m = v->mass[v->pid[i]];
    const float *x = v->vel + 3 * v->pid[i];
    msum += m;
    svx += x[0] * m;
    svy += x[1] * m;
    svz += x[2] * m;
  }
  cov[0] = (float)(svx / msum);
  cov[1] = (float)(svy / msum);
  cov[2] = (float)(svz / msum);
  return msum;
}

/* EnergySnapshot_t::AveragePosition, subhalo_unbind.cpp:139-188 */
static void average_position(const eview *v, int64_t num, float com[3], const dpar *d, int nthr)
{
  double sx = 0., sy = 0., sz = 0., msum = 0., origin[3] = {0., 0., 0.};
  if (num == 0) return;
  if (num == 1) {
    memcpy(com, v->pos + 3 * v->pid[0], 3 * sizeof(float));
    return;
  }
  if (d->periodic)
    for (int j = 0; j < 3; j++) origin[j] = v->pos[3 * v->pid[0] + j];
#pragma omp parallel for reduction(+ : msum, sx, sy, sz) if (num > 100) num_threads(nthr)
  for (int64_t i = 0; i < num; i++) {
    const float m = v->mass[v->pid[i]];
    const float *x = v->pos + 3 * v->pid[i];
    msum += m;
    if (d->periodic) {
      sx += nearest_d(x[0] - origin[0], d) * m;
      sy += nearest_d(x[1] - origin[1], d) * m;
      sz += nearest_d(x[2] - origin[2], d) * m;
    } else {
      sx += x[0] * m; /* float products, as in the reference */
      sy += x[1] * m;
      sz += x[2] * m;
    }
  }
  sx /= msum;
  sy /= msum;
  sz /= msum;
  if (d->periodic) {
    sx += origin[0];
    sy += origin[1];
    sz += origin[2];
  }
  com[0] = (float)sx;
  com[1] = (float)sy;
  com[2] = (float)sz;
}

/* EnergySnapshot_t::AverageKinematics, subhalo_unbind.cpp:189-232 */
static void average_kinematics(const eview *v, int64_t num, const float rp[3], const float rv[3],
                               const dpar *d, hbto_result *res, int nthr)
{
  double E = 0., K = 0., AMx = 0., AMy = 0., AMz = 0., M = 0.;
  if (num <= 1) {
    res->specific_potential = 0.f;
    res->specific_kinetic = 0.f;
    res->specific_angmom[0] = res->specific_angmom[1] = res->specific_angmom[2] = 0.f;
    return;
  }
#pragma omp parallel for reduction(+ : E, K, AMx, AMy, AMz, M) if (num > 100) num_threads(nthr)
  for (int64_t i = 0; i < num; i++) {
    const float m = v->mass[v->pid[i]];
    const float *x = v->pos + 3 * v->pid[i];
    const float *u = v->vel + 3 * v->pid[i];
    double dx[3], dv[3];
    E += v->E[i] * m; /* float product */
    for (int j = 0; j < 3; j++) {
      dx[j] = x[j] - rp[j]; /* float difference */
      if (d->periodic) dx[j] = nearest_d(dx[j], d);
      dx[j] *= d->a;
      dv[j] = (u[j] - rv[j]) + d->Hz * dx[j];
      K += dv[j] * dv[j] * m;
    }
    AMx += (dx[1] * dv[2] - dx[2] * dv[1]) * m;
    AMy += (dx[2] * dv[0] - dx[0] * dv[2]) * m;
    AMz += (dx[0] * dv[1] - dx[1] * dv[0]) * m;
    M += m;
  }
  E /= M;
  K *= 0.5 / M;
  res->specific_potential = (float)(E - K);
  res->specific_kinetic = (float)K;
  res->specific_angmom[0] = (float)(AMx / M);
  res->specific_angmom[1] = (float)(AMy / M);
  res->specific_angmom[2] = (float)(AMz / M);
}

/* Subhalo_t::CountParticleTypes, src/subhalo.cpp:400-444 (serial form).
 * The reference's serial branch (Nbound<=100) skips NullParticleId entries. */
static void count_types(const int64_t *order, int64_t nbound, const int64_t *id, const float *mass,
                        const int32_t *type, hbto_result *res)
{
  for (int k = 0; k < 6; k++) {
    res->nbound_type[k] = 0;
    res->mbound_type[k] = 0.f;
  }
  for (int64_t i = 0; i < nbound; i++) {
    int64_t p = order[i];
    int t = type ? type[p] : 1;
    if (nbound <= 100 && id[p] == -1) continue;
    if (t < 0 || t > 5) continue;
    res->nbound_type[t]++;
    res->mbound_type[t] += mass[p];
  }
}

/* Subhalo_t::CountParticles, src/subhalo.cpp:479-499 (N==0 and N==1 exits) */
static void count_particles(const int64_t *order, int64_t nbound, const int64_t *id,
                            const float *mass, const int32_t *type, hbto_result *res)
{
  (void)id;
  for (int k = 0; k < 6; k++) {
    res->nbound_type[k] = 0;
    res->mbound_type[k] = 0.f;
  }
  for (int64_t i = 0; i < nbound; i++) {
    int t = type ? type[order[i]] : 1;
    if (t < 0 || t > 5) continue;
    res->nbound_type[t]++;
    res->mbound_type[t] += mass[order[i]];
  }
  float m = 0.f;
  for (int k = 0; k < 6; k++) m += res->mbound_type[k];
  res->mbound = m;
}

/* ------------------------------------------------------------------------ */
/* RefineBindingEnergyOrder, subhalo_unbind.cpp:234-262 */
static void refine_order(otree *t, float *E, int64_t *pid, int64_t size, const float *pos,
                         const float *vel, const float *mass, const float rp[3], const float rv[3],
                         const dpar *d, int nthr, int64_t *cnt)
{
  float *Ei = malloc(size * sizeof(float));
  int64_t *pi = malloc(size * sizeof(int64_t));
  float *E2 = malloc(size * sizeof(float));
  int64_t *p2 = malloc(size * sizeof(int64_t));
  int64_t c = 0;
  tree_build(t, pid, size, pos, mass, 1.f, d);
#pragma omp parallel for reduction(+ : c) if (size > 100) num_threads(nthr)
  for (int64_t i = 0; i < size; i++) {
    int64_t p = pid[i];
    pi[i] = i;
    Ei[i] = (float)binding_energy(t, pos + 3 * p, vel + 3 * p, rp, rv, mass[p], d, &c);
  }
  *cnt += c;
  sort_energy_alloc(Ei, pi, size);
  for (int64_t i = 0; i < size; i++) {
    E2[i] = E[pi[i]];
    p2[i] = pid[pi[i]];
  }
  memcpy(E, E2, size * sizeof(float));
  memcpy(pid, p2, size * sizeof(int64_t));
  free(Ei);
  free(pi);
  free(E2);
  free(p2);
}

#define HBTO_MAX_PASSES 100000

/* Subhalo_t::Unbind, src/subhalo_unbind.cpp:263-431 */
static int unbind_one(const dpar *d, int64_t n, const int64_t *id, const float *pos,
                      const float *vel, const float *mass, const int32_t *type,
                      const hbto_state *st, int64_t *order, float *energy, hbto_result *res,
                      int nthr)
{
  memset(res, 0, sizeof(*res));
  random_splits = 0;
  memcpy(res->ref_pos, st->ref_pos, sizeof(res->ref_pos));
  memcpy(res->ref_vel, st->ref_vel, sizeof(res->ref_vel));
  memcpy(res->mostbound_pos, st->mostbound_pos, sizeof(res->mostbound_pos));
  memcpy(res->mostbound_vel, st->mostbound_vel, sizeof(res->mostbound_vel));
  for (int64_t i = 0; i < n; i++) {
    order[i] = i;
    energy[i] = NAN;
  }
  res->too_few = (n < d->minpart); /* :269-273 */
  if (n == 0) {                    /* :275-283 */
    res->nbound = 0;
    count_particles(order, 0, id, mass, type, res);
    return 0;
  }
  if (n == 1) { /* :284-293 */
    res->nbound = 1;
    count_particles(order, 1, id, mass, type, res);
    energy[0] = 0.f;
    return 0;
  }

  int64_t S = d->maxsample;
  float RefPos[3], RefVel[3], OldRefPos[3] = {0, 0, 0}, OldRefVel[3] = {0, 0, 0};
  memcpy(RefPos, st->ref_pos, sizeof(RefPos));
  memcpy(RefVel, st->ref_vel, sizeof(RefVel));
  int64_t Nbound = n, Nlast = n;
  float *E = malloc(n * sizeof(float));
  int64_t *pid = malloc(n * sizeof(int64_t));
  for (int64_t i = 0; i < n; i++) {
    pid[i] = i;
    E[i] = 0.f;
  }
  otree tree;
  tree_init(&tree);
  int correction = 0, passes = 0, rc = 0;
  int64_t cnt = 0, evals = 0;
  eview ev = {pos, vel, mass, pid, E};

  for (;;) {
    if (++passes > HBTO_MAX_PASSES) {
      rc = -2;
      break;
    }
    if (correction) { /* :312-330 */
      float dV[3];
      relvel(OldRefPos, OldRefVel, RefPos, RefVel, dV, d);
      const float dK = (float)(0.5 * (dV[0] * dV[0] + dV[1] * dV[1] + dV[2] * dV[2]));
      tree_build(&tree, pid + Nbound, Nlast - Nbound, pos, mass, 1.f, d);
      int64_t c = 0;
#pragma omp parallel for reduction(+ : c) if (Nlast > 100) num_threads(nthr)
      for (int64_t i = 0; i < Nbound; i++) {
        const int64_t p = pid[i];
        const float *x = pos + 3 * p, *v = vel + 3 * p;
        float ov[3];
        relvel(x, v, OldRefPos, OldRefVel, ov, d);
        const float t = (ov[0] * dV[0] + ov[1] * dV[1] + ov[2] * dV[2]) + dK;
        E[i] = (float)((double)E[i] + ((double)t - eval_potential(&tree, x, 0.f, d, &c)));
      }
      cnt += c;
      evals += Nbound;
      Nlast = Nbound;
    } else { /* :331-356 */
      Nlast = Nbound;
      int64_t np_tree = Nlast;
      float mf = 1.f;
      if (S > 0 && Nlast > S) {
        np_tree = S;
        mf = (float)Nlast / (float)S;
      }
      tree_build(&tree, pid, np_tree, pos, mass, mf, d);
      int64_t c = 0;
#pragma omp parallel for reduction(+ : c) if (Nlast > 100) num_threads(nthr)
      for (int64_t i = 0; i < Nlast; i++) {
        const int64_t p = pid[i];
        const float m = (i < np_tree) ? mass[p] * mf : 0.f;
        E[i] = (float)binding_energy(&tree, pos + 3 * p, vel + 3 * p, RefPos, RefVel, m, d, &c);
      }
      cnt += c;
      evals += Nlast;
    }
    Nbound = partition_energy(E, pid, Nlast); /* :357 */
    if (Nbound < d->minpart) {                /* disruption, :361-379 */
      Nbound = 1;
      Nlast = 1;
      res->disrupted = 1;
      for (int64_t k = 0; k < n; k++) {
        if (id[order[k]] == st->mostbound_id) {
          int64_t tmp = order[k];
          order[k] = order[0];
          order[0] = tmp;
          break;
        }
      }
      memcpy(RefPos, st->mostbound_pos, sizeof(RefPos));
      memcpy(RefVel, st->mostbound_vel, sizeof(RefVel));
      res->mbound = mass[order[0]];
      energy[0] = E[0];
      break;
    }
    sort_energy_alloc(E + Nbound, pid + Nbound, Nlast - Nbound); /* :382 */
    {
      int64_t Ndiff = Nlast - Nbound;
      if (Ndiff < Nbound) {
        if (S <= 0 || Ndiff < S) {
          correction = 1;
          memcpy(OldRefPos, RefPos, sizeof(RefPos));
          memcpy(OldRefVel, RefVel, sizeof(RefVel));
        }
      }
    }
    res->mbound = (float)average_velocity(&ev, Nbound, RefVel, nthr); /* :393 */
    average_position(&ev, Nbound, RefPos, d, nthr);                    /* :394 */
    if ((float)Nbound >= (float)Nlast * d->prec) {                     /* :395 */
      res->converged = 1;
      sort_energy_alloc(E, pid, Nbound); /* :405 */
      if (d->refine && Nbound > S) { /* :406-407 */
        refine_order(&tree, E, pid, S, pos, vel, mass, RefPos, RefVel, d, nthr, &cnt);
        evals += S;
      }
      for (int64_t i = 0; i < n; i++) { /* :409-415 */
        order[i] = pid[i];
        energy[i] = E[i];
        pid[i] = i;
      }
      break;
    }
  }
  res->nbound = Nbound;
  res->iterations = passes;
  res->evaluations = evals;
  res->interactions = cnt;
  memcpy(res->ref_pos, RefPos, sizeof(RefPos));
  memcpy(res->ref_vel, RefVel, sizeof(RefVel));
  if (res->converged) { /* :417-418 */
    memcpy(res->mostbound_pos, pos + 3 * order[0], 3 * sizeof(float));
    memcpy(res->mostbound_vel, vel + 3 * order[0], 3 * sizeof(float));
    /* AverageKinematics over the permuted list: Elist[i].pid == i (:423) */
    int64_t *po = malloc(n * sizeof(int64_t));
    for (int64_t i = 0; i < n; i++) po[i] = order[i];
    eview fin = {pos, vel, mass, po, energy};
    average_kinematics(&fin, Nbound, RefPos, RefVel, d, res, nthr);
    free(po);
  } else {
    average_kinematics(&ev, Nbound, RefPos, RefVel, d, res, nthr);
  }
  count_types(order, Nbound, id, mass, type, res); /* :424 */
  tree_free(&tree);
  free(E);
  free(pid);
  res->random_splits = random_splits;
  return rc;
}

int hbto_unbind(const hbto_params *par, int64_t n, const int64_t *id, const float *pos,
                const float *vel, const float *mass, const int32_t *type, const hbto_state *st,
                int64_t *order, float *energy, hbto_result *res, int nthreads)
{
  dpar d;
  derive(par, &d);
#ifdef _OPENMP
  int nthr = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nthr = 1;
  (void)nthreads;
#endif
  return unbind_one(&d, n, id, pos, vel, mass, type, st, order, energy, res, nthr);
}

int hbto_unbind_batch(const hbto_params *par, int64_t nsub, const int64_t *off, const int64_t *id,
                      const float *pos, const float *vel, const float *mass, const int32_t *type,
                      const hbto_state *st, int64_t *order, float *energy, hbto_result *res,
                      int nthreads)
{
  dpar d;
  int rc = 0;
  derive(par, &d);
#ifdef _OPENMP
  int nthr = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nthr = 1;
  (void)nthreads;
#endif
  /* halo-parallel; inner particle loops run serially (nesting is off, HBT.cpp:22) */
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthr) reduction(| : rc)
  for (int64_t s = 0; s < nsub; s++) {
    const int64_t o = off[s], m = off[s + 1] - off[s];
    rc |= unbind_one(&d, m, id + o, pos + 3 * o, vel + 3 * o, mass + o, type ? type + o : NULL,
                     st + s, order + o, energy + o, res + s, 1);
  }
  return rc;
}

int hbto_binding_energies(const hbto_params *par, int64_t n, const float *pos, const float *vel,
                          const float *mass, const float ref_pos[3], const float ref_vel[3],
                          float *energy, double *potential, int64_t *interactions, int nthreads)
{
  dpar d;
  derive(par, &d);
#ifdef _OPENMP
  int nthr = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nthr = 1;
  (void)nthreads;
#endif
  int64_t *pid = malloc((n > 0 ? n : 1) * sizeof(int64_t)), c = 0;
  for (int64_t i = 0; i < n; i++) pid[i] = i;
  otree t;
  tree_init(&t);
  tree_build(&t, pid, n, pos, mass, 1.f, &d);
#pragma omp parallel for reduction(+ : c) if (n > 100) num_threads(nthr)
  for (int64_t i = 0; i < n; i++) {
    double pot = eval_potential(&t, pos + 3 * i, mass[i], &d, &c);
    float dv[3];
    relvel(pos + 3 * i, vel + 3 * i, ref_pos, ref_vel, dv, &d);
    if (potential) potential[i] = pot;
    energy[i] = (float)((dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]) * 0.5 + pot);
  }
  if (interactions) *interactions = c;
  tree_free(&t);
  free(pid);
  return 0;
}

/* The potentials GravityTree_t::EvaluatePotential (src/gravity_tree.cpp:79-164)
 * gives the particles targets[0..ntarget) from one tree over all n particles
 * (OctTree_t::Build + UpdateInternalNodes, src/oct_tree.tpp:16-144,
 * src/gravity_tree.cpp:18-77), self term cancelled as in the first pass of the
 * loop (src/subhalo_unbind.cpp:341-354), for each of ntheta opening angles:
 * the tree does not depend on the angle, so it is built once.
 * potential[k*ntarget + j] is target j at open_angles[k]; interactions[k]
 * (may be NULL) counts the contributions summed at that angle. */
int hbto_tree_potentials(const hbto_params *par, int64_t n, const float *pos, const float *mass,
                         int64_t ntarget, const int64_t *targets, int32_t ntheta,
                         const double *open_angles, double *potential, int64_t *interactions,
                         int nthreads)
{
  dpar d;
  derive(par, &d);
#ifdef _OPENMP
  int nthr = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nthr = 1;
  (void)nthreads;
#endif
  for (int64_t j = 0; j < ntarget; j++)
    if (targets[j] < 0 || targets[j] >= n) return 1;
  int64_t *pid = malloc((n > 0 ? n : 1) * sizeof(int64_t));
  if (!pid) return 2;
  for (int64_t i = 0; i < n; i++) pid[i] = i;
  otree t;
  tree_init(&t);
  tree_build(&t, pid, n, pos, mass, 1.f, &d);
  for (int32_t k = 0; k < ntheta; k++) {
    hbto_params pk = *par;
    pk.open_angle = open_angles[k];
    dpar dk;
    derive(&pk, &dk);
    int64_t c = 0;
#pragma omp parallel for reduction(+ : c) schedule(dynamic, 64) num_threads(nthr)
    for (int64_t j = 0; j < ntarget; j++) {
      const int64_t i = targets[j];
      potential[(size_t)k * ntarget + j] = eval_potential(&t, pos + 3 * i, mass[i], &dk, &c);
    }
    if (interactions) interactions[k] = c;
  }
  tree_free(&t);
  free(pid);
  return 0;
}

void hbto_srand48(long seed) { srand48(seed); }

/* ------------------------------------------------------------------ ID tables */

typedef struct {
  int64_t key, pos;
} keypos;

static int cmp_keypos(const void *a, const void *b)
{
  const keypos *x = (const keypos *)a, *y = (const keypos *)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return x->pos < y->pos ? -1 : (x->pos > y->pos); /* first in input order first */
}

/* MappedIndexTable_t::Fill (hash.tpp:18-30): the (key, index) pairs sorted by
 * key; GetIndex (hash.tpp:47-55): a negative key is absent, else binary search. */
static void mapped_lookup(const int64_t *keys, const int64_t *values, int64_t n, int64_t null_index,
                          const int64_t *queries, int64_t m, int64_t *out)
{
  keypos *map = malloc((n > 0 ? n : 1) * sizeof(keypos));
  for (int64_t i = 0; i < n; i++) {
    map[i].key = keys[i];
    map[i].pos = i;
  }
  qsort(map, (size_t)n, sizeof(keypos), cmp_keypos);
  for (int64_t j = 0; j < m; j++) {
    const int64_t q = queries[j];
    out[j] = null_index;
    if (q < 0) continue;
    int64_t lo = 0, hi = n; /* lower_bound */
    while (lo < hi) {
      const int64_t mid = lo + (hi - lo) / 2;
      if (map[mid].key < q)
        lo = mid + 1;
      else
        hi = mid;
    }
    if (lo < n && map[lo].key == q) out[j] = values[map[lo].pos];
  }
  free(map);
}

/* FlatIndexTable_t::Fill (hash.tpp:59-95): a dense array over [KeyMin, KeyMax]
 * set to null, then Index[key] = index for every pair; GetIndex
 * (hash.tpp:104-109): null outside [KeyMin, KeyMax]. */
static void flat_lookup(const int64_t *keys, const int64_t *values, int64_t n, int64_t null_index,
                        const int64_t *queries, int64_t m, int64_t *out)
{
  if (n == 0) {
    for (int64_t j = 0; j < m; j++) out[j] = null_index;
    return;
  }
  int64_t kmin = keys[0], kmax = keys[0];
  for (int64_t i = 1; i < n; i++) {
    if (keys[i] > kmax) kmax = keys[i];
    if (keys[i] < kmin) kmin = keys[i];
  }
  const int64_t span = kmax - kmin + 1;
  int64_t *index = malloc((size_t)span * sizeof(int64_t));
  for (int64_t k = 0; k < span; k++) index[k] = null_index;
  for (int64_t i = 0; i < n; i++) index[keys[i] - kmin] = values[i];
  for (int64_t j = 0; j < m; j++) {
    const int64_t q = queries[j];
    out[j] = (q < kmin || q > kmax) ? null_index : index[q - kmin];
  }
  free(index);
}

int hbto_index_lookup(int flat, const int64_t *keys, const int64_t *values, int64_t n,
                      int64_t null_index, const int64_t *queries, int64_t m, int64_t *out)
{
  if (n < 0 || m < 0) return -1;
  if (flat)
    flat_lookup(keys, values, n, null_index, queries, m, out);
  else
    mapped_lookup(keys, values, n, null_index, queries, m, out);
  return 0;
}

/* ------------------------------------------------------------ properties */

typedef struct {
  float r, m, v;
  int64_t k;
} radmass;

static int cmp_radmass(const void *a, const void *b)
{
  const radmass *x = (const radmass *)a, *y = (const radmass *)b;
  if (x->r != y->r) return x->r < y->r ? -1 : 1;
  return x->k < y->k ? -1 : (x->k > y->k); /* ties keep the given order */
}

int hbto_subhalo_properties(const hbto_params *par, int64_t nbound, const float *pos,
                            const float *mass, const float cen[3], float mbound,
                            float last_max_vmax, int32_t last_snap, int32_t snapshot_index,
                            hbto_props *out)
{
  dpar d;
  derive(par, &d);
  memset(out, 0, sizeof(*out));
  out->last_max_vmax_physical = last_max_vmax;
  out->snapshot_of_last_max_vmax = last_snap;
  if (nbound <= 1) return 0; /* subhalo.cpp:264-282, :339-351 */
  const float G = (float)par->G, a = (float)par->scale_factor, Hz = (float)par->hubble;
  const float eps = (float)par->softening;
  /* CalculateProfileProperties (subhalo.cpp:283-312): distances to the most-bound
   * particle (PeriodicDistance, config_parser.h:143-156), sorted, cumulative mass
   * in double, radius floored at the softening, v^2 = m / r */
  const float VelocityUnit = G / a;
  radmass *prof = malloc((size_t)nbound * sizeof(radmass));
  for (int64_t i = 0; i < nbound; i++) {
    float dx[3];
    for (int j = 0; j < 3; j++) {
      dx[j] = pos[3 * i + j] - cen[j];
      if (d.periodic) dx[j] = nearest_f(dx[j], &d);
    }
    prof[i].r = sqrtf(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
    prof[i].m = mass[i];
    prof[i].k = i;
  }
  qsort(prof, (size_t)nbound, sizeof(radmass), cmp_radmass);
  double m_cum = 0.;
  for (int64_t i = 0; i < nbound; i++) prof[i].m = (float)(m_cum += prof[i].m);
  for (int64_t i = 0; i < nbound; i++) {
    if (prof[i].r < eps) prof[i].r = eps;
    prof[i].v = prof[i].m / prof[i].r;
  }
  int64_t imax = 0;
  for (int64_t i = 1; i < nbound; i++)
    if (prof[i].v > prof[imax].v) imax = i; /* max_element: the first maximum */
  out->rmax_comoving = prof[imax].r;
  out->vmax_physical = sqrtf(prof[imax].v * VelocityUnit);
  out->rhalf_comoving = prof[nbound / 2].r;
  out->r2sigma_comoving = prof[(int64_t)(nbound * 0.955)].r;
  /* SphericalOverdensitySize with virialF_c200 = 200 (snapshot.cpp:259-281, :328-336) */
  const float RhoVirial = (float)((double)(200.f * Hz * Hz) / 2.0 / (double)G * (double)a *
                                  (double)a * (double)a);
  for (int64_t i = nbound - 1; i >= 0; i--) {
    const float r = prof[i].r, m = prof[i].m;
    if (m > RhoVirial * r * r * r) {
      out->m200crit = m;
      out->r200crit_comoving = (float)pow((double)(m / RhoVirial), 1.0 / 3);
      break;
    }
  }
  if (out->vmax_physical >= last_max_vmax) { /* subhalo.cpp:314-318 */
    out->snapshot_of_last_max_vmax = snapshot_index;
    out->last_max_vmax_physical = out->vmax_physical;
  }
  free(prof);
  /* CalculateShape (subhalo.cpp:352-392): float terms summed in double over the
   * bound particles after the most-bound one */
  double I[6] = {0, 0, 0, 0, 0, 0}, W[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t i = 1; i < nbound; i++) {
    const float m = mass[i];
    float dx = pos[3 * i] - cen[0], dy = pos[3 * i + 1] - cen[1], dz = pos[3 * i + 2] - cen[2];
    if (d.periodic) {
      dx = nearest_f(dx, &d);
      dy = nearest_f(dy, &d);
      dz = nearest_f(dz, &d);
    }
    const float dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
    I[0] += dx2 * m;
    I[3] += dy2 * m;
    I[5] += dz2 * m;
    I[1] += dx * dy * m;
    I[2] += dx * dz * m;
    I[4] += dy * dz * m;
    float dr2 = dx2 + dy2 + dz2;
    dr2 /= m;
    W[0] += dx2 / dr2;
    W[3] += dy2 / dr2;
    W[5] += dz2 / dr2;
    W[1] += dx * dy / dr2;
    W[2] += dx * dz / dr2;
    W[4] += dy * dz / dr2;
  }
  for (int k = 0; k < 6; k++) {
    out->inertial_tensor[k] = (float)I[k] / mbound;
    out->inertial_tensor_weighted[k] = (float)W[k] / mbound;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Merging: SubHelper_t::BuildPosition / BuildVelocity, SinkDistance and
 * DetectTraps (src/subhalo_merge.cpp:30-165).                               */
#define CORE_PARTICLES 20 /* NumPartCoreMax, subhalo_merge.cpp:11 */
#define DELTA_CRIT 2.f    /* DeltaCrit, :12 */

static void build_core(const dpar *d, int64_t nb, const float *pos, const float *vel,
                       const float *mass, hbto_core *c)
{
  memset(c, 0, sizeof(*c));
  if (nb <= 0) return; /* :32-36, :83-87 (position left unset there) */
  if (nb == 1) {       /* :37-42, :88-93 */
    for (int j = 0; j < 3; j++) {
      c->pos[j] = pos[j];
      c->vel[j] = vel[j];
    }
    return;
  }
  const int64_t np = nb > CORE_PARTICLES ? CORE_PARTICLES : nb;
  double sx[3] = {0, 0, 0}, sx2[3] = {0, 0, 0}, origin[3] = {0, 0, 0}, msum = 0.;
  if (d->periodic)
    for (int j = 0; j < 3; j++) origin[j] = pos[j];
  for (int64_t i = 0; i < np; i++) { /* :55-70 */
    const float m = mass[i];
    msum += m;
    for (int j = 0; j < 3; j++) {
      double dx;
      if (d->periodic)
        dx = nearest_d((double)pos[3 * i + j] - origin[j], d);
      else
        dx = pos[3 * i + j];
      sx[j] += dx * m;
      sx2[j] += dx * dx * m;
    }
  }
  for (int j = 0; j < 3; j++) { /* :72-80 */
    sx[j] /= msum;
    sx2[j] /= msum;
    c->pos[j] = (float)sx[j];
    if (d->periodic) c->pos[j] = (float)((double)c->pos[j] + origin[j]);
    sx2[j] -= sx[j] * sx[j];
  }
  c->sigma_r = (float)sqrt(sx2[0] + sx2[1] + sx2[2]);
  double sv[3] = {0, 0, 0}, sv2[3] = {0, 0, 0};
  msum = 0.;
  for (int64_t i = 0; i < np; i++) { /* :104-116 */
    const float m = mass[i];
    msum += m;
    for (int j = 0; j < 3; j++) {
      const double dv = vel[3 * i + j];
      sv[j] += dv * m;
      sv2[j] += dv * dv * m;
    }
  }
  for (int j = 0; j < 3; j++) { /* :118-124 */
    sv[j] /= msum;
    sv2[j] /= msum;
    c->vel[j] = (float)sv[j];
    sv2[j] -= sv[j] * sv[j];
  }
  c->sigma_v = (float)sqrt(sv2[0] + sv2[1] + sv2[2]);
}

/* SinkDistance (:128-133) with PeriodicDistance (config_parser.h:143-156)
 * and Distance (mymath.h:184-187), in float. */
static float sink_distance(const dpar *d, const float *mbp, const float *mbv, const hbto_core *c)
{
  float dx[3], dv[3];
  for (int j = 0; j < 3; j++) {
    dx[j] = c->pos[j] - mbp[j];
    if (d->periodic) dx[j] = nearest_f(dx[j], d);
    dv[j] = c->vel[j] - mbv[j];
  }
  const float r = sqrtf(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
  const float v = sqrtf(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
  return r / c->sigma_r + v / c->sigma_v;
}

int hbto_merge_detect(const hbto_params *par, int64_t nsub, const int64_t *list_off,
                      const float *pos, const float *vel, const float *mass,
                      const int64_t *nbound, const int64_t *host, const float *mb_pos,
                      const float *mb_vel, int32_t isnap, int64_t *sink, int32_t *sink_snap,
                      int32_t *merged, hbto_core *cores)
{
  dpar d;
  derive(par, &d);
  hbto_core *c = malloc((size_t)(nsub > 0 ? nsub : 1) * sizeof(hbto_core));
  for (int64_t s = 0; s < nsub; s++) { /* FillCores, :172-180 */
    const int64_t o = list_off[s];
    int64_t nb = nbound[s];
    if (nb > list_off[s + 1] - o) nb = list_off[s + 1] - o;
    build_core(&d, nb, pos + 3 * o, vel + 3 * o, mass + o, c + s);
  }
  int rc = 0;
  for (int64_t s = 0; s < nsub; s++) { /* DetectTraps, :135-160 */
    if (sink[s] >= 0) continue;       /* IsTrapped */
    int64_t h = host[s], steps = 0;
    while (h >= 0) {
      if (++steps > nsub) {
        rc = -1;
        break;
      }
      if (nbound[h] > 1 && sink_distance(&d, mb_pos + 3 * s, mb_vel + 3 * s, c + h) < DELTA_CRIT) {
        sink[s] = h;
        sink_snap[s] = isnap;
        if (nbound[s] > 1) merged[h] = 1;
        break;
      }
      h = host[h];
    }
  }
  if (cores) memcpy(cores, c, (size_t)nsub * sizeof(hbto_core));
  free(c);
  return rc;
}
