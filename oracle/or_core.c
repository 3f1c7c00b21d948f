/*
 * or_core.c -- oracle (test infrastructure): transforms, AABBs, geometry
 * closing (daughter AABBs, BVHs, navigation index table).
 */
#include <stdio.h>

#include "or_internal.h"

/* ------------------------------------------------------------------ */
/* Transformation3D                                                    */
/* ------------------------------------------------------------------ */

/* default constructor, Transformation3D.h:67-69 */
void xf_identity(or_xf *m)
{
  memset(m, 0, sizeof(*m));
  m->r[0] = m->r[4] = m->r[8] = 1.;
  m->identity = 1;
}

/* Transformation3D(tx,ty,tz,r0..r8) -> SetTranslation, SetRotation, SetProperties
 * (source/Transformation3D.cpp:52-61, 117-126, 170-182) */
void xf_from12(or_xf *m, const double *a)
{
  int i, code = 0;
  for (i = 0; i < 3; ++i) m->t[i] = a[i];
  for (i = 0; i < 9; ++i) m->r[i] = a[3 + i];
  m->has_trans = (fabs(m->t[0]) > kTolerance || fabs(m->t[1]) > kTolerance || fabs(m->t[2]) > kTolerance) ? 1 : 0;
  for (i = 0; i < 9; ++i) code |= (1 << i) * (fabs(m->r[i]) > kTolerance);
  if (code == 0x111 && (m->r[0] == 1. && m->r[4] == 1. && m->r[8] == 1.)) code = 0x200;
  m->has_rot  = (code == 0x200) ? 0 : 1;
  m->identity = !m->has_trans && !m->has_rot;
}

/* Transform<kGeneric,kGeneric>: DoTranslation then the general DoRotation
 * (Transformation3D.h:663-673, 729-735, 746-770) */
v3 xf_transform(const or_xf *m, v3 p)
{
  double t0 = p.x - m->t[0], t1 = p.y - m->t[1], t2 = p.z - m->t[2];
  double l0, l1, l2;
  l0 = t0 * m->r[0];
  l1 = t0 * m->r[1];
  l2 = t0 * m->r[2];
  l0 += t1 * m->r[3];
  l1 += t1 * m->r[4];
  l2 += t1 * m->r[5];
  l0 += t2 * m->r[6];
  l1 += t2 * m->r[7];
  l2 += t2 * m->r[8];
  return v3_make(l0, l1, l2);
}

/* TransformDirection<kGeneric> (Transformation3D.h:959-975) */
v3 xf_transform_dir(const or_xf *m, v3 d)
{
  double l0, l1, l2;
  l0 = d.x * m->r[0];
  l1 = d.x * m->r[1];
  l2 = d.x * m->r[2];
  l0 += d.y * m->r[3];
  l1 += d.y * m->r[4];
  l2 += d.y * m->r[5];
  l0 += d.z * m->r[6];
  l1 += d.z * m->r[7];
  l2 += d.z * m->r[8];
  return v3_make(l0, l1, l2);
}

/* InverseTransformKernel<false> (Transformation3D.h:793-827) */
v3 xf_inverse_transform(const or_xf *m, v3 l)
{
  double a, b, c;
  a = m->t[0];
  a += l.x * m->r[0];
  a += l.y * m->r[1];
  a += l.z * m->r[2];
  b = m->t[1];
  b += l.x * m->r[3];
  b += l.y * m->r[4];
  b += l.z * m->r[5];
  c = m->t[2];
  c += l.x * m->r[6];
  c += l.y * m->r[7];
  c += l.z * m->r[8];
  return v3_make(a, b, c);
}

/* MultiplyFromRight (Transformation3D.h:878-946) */
void xf_multiply_from_right(or_xf *m, const or_xf *rhs)
{
  double tx, ty, tz;
  if (rhs->identity) return;
  m->identity = 0;
  if (rhs->has_trans) {
    m->has_trans = 1;
    m->t[0] += m->r[0] * rhs->t[0];
    m->t[0] += m->r[1] * rhs->t[1];
    m->t[0] += m->r[2] * rhs->t[2];
    m->t[1] += m->r[3] * rhs->t[0];
    m->t[1] += m->r[4] * rhs->t[1];
    m->t[1] += m->r[5] * rhs->t[2];
    m->t[2] += m->r[6] * rhs->t[0];
    m->t[2] += m->r[7] * rhs->t[1];
    m->t[2] += m->r[8] * rhs->t[2];
  }
  if (rhs->has_rot) {
    int row;
    m->has_rot = 1;
    for (row = 0; row < 3; ++row) {
      double *r = m->r + 3 * row;
      tx   = r[0];
      ty   = r[1];
      tz   = r[2];
      r[0] = tx * rhs->r[0];
      r[1] = tx * rhs->r[1];
      r[2] = tx * rhs->r[2];
      r[0] += ty * rhs->r[3];
      r[1] += ty * rhs->r[4];
      r[2] += ty * rhs->r[5];
      r[0] += tz * rhs->r[6];
      r[1] += tz * rhs->r[7];
      r[2] += tz * rhs->r[8];
    }
  }
}

/* ------------------------------------------------------------------ */
/* AABB                                                                */
/* ------------------------------------------------------------------ */

/* AABB::ComputeIntersectionInvDir (AABB.h:136-154) */
void aabb_intersect_invdir(const or_aabb *b, v3 p, v3 invdir, double *tmin, double *tmax)
{
  v3 t0 = v3_mul(v3_sub(b->mn, p), invdir);
  v3 t1 = v3_mul(v3_sub(b->mx, p), invdir);
  double s;
  if (t0.x > t1.x) { s = t0.x; t0.x = t1.x; t1.x = s; }
  if (t0.y > t1.y) { s = t0.y; t0.y = t1.y; t1.y = s; }
  if (t0.z > t1.z) { s = t0.z; t0.z = t1.z; t1.z = s; }
  *tmin = v3_maxc(t0);
  *tmax = v3_minc(t1) * (1. + 2 * kEpsilon);
}

/* ------------------------------------------------------------------ */
/* geometry closing                                                    */
/* ------------------------------------------------------------------ */

static void set_err(char *err, int errlen, const char *msg)
{
  if (err && errlen > 0) snprintf(err, (size_t)errlen, "%s", msg);
}

/* ABBoxManager::ComputeABBox (source/ABBoxManager.cpp:109-142) */
static void compute_abbox(const or_geom *g, int pv, or_aabb *out)
{
  const or_lv *lv = &g->lv[g->pv[pv].lv];
  v3 lower, upper, delta;
  double minx = kInfLength, miny = kInfLength, minz = kInfLength;
  double maxx = -kInfLength, maxy = -kInfLength, maxz = -kInfLength;
  int x, y, z;
  shape_extent(lv, &lower, &upper);
  delta = v3_sub(upper, lower);
  for (x = 0; x <= 1; ++x)
    for (y = 0; y <= 1; ++y)
      for (z = 0; z <= 1; ++z) {
        v3 corner, tc;
        corner.x = lower.x + x * delta.x;
        corner.y = lower.y + y * delta.y;
        corner.z = lower.z + z * delta.z;
        tc       = xf_inverse_transform(&g->pv[pv].xf, corner);
        minx     = tc.x < minx ? tc.x : minx; /* std::min(minx, v) */
        miny     = tc.y < miny ? tc.y : miny;
        minz     = tc.z < minz ? tc.z : minz;
        maxx     = maxx < tc.x ? tc.x : maxx; /* std::max(maxx, v) */
        maxy     = maxy < tc.y ? tc.y : maxy;
        maxz     = maxz < tc.z ? tc.z : maxz;
      }
  out->mn = v3_make(minx - 1E-3, miny - 1E-3, minz - 1E-3);
  out->mx = v3_make(maxx + 1E-3, maxy + 1E-3, maxz + 1E-3);
}

/* ---- navigation index table (source/NavIndexTable.cpp:9-99,
 *      VecGeom/management/NavIndexTable.h:114-176) ---- */
typedef struct {
  int count;            /* counting pass */
  size_t table_bytes;   /* fTableSize, starts at sizeof(NavIndex_t) */
  uint32_t current;     /* fCurrent, starts at 1 */
  uint32_t *tab;
  int path[64];         /* placed-volume ids from the world down */
} nav_visitor;

static uint32_t nav_apply(const or_geom *g, nav_visitor *v, int level, uint32_t mother, int dind)
{
  int pv              = v->path[level];
  const or_lv *lv     = &g->lv[g->pv[pv].lv];
  unsigned short nd   = (unsigned short)lv->nd;
  uint32_t new_mother = v->current;
  size_t before       = v->count ? v->table_bytes / 4 : v->current;
  uint32_t dindices   = 3 + nd + ((nd + 1) & 1);
  int pad             = ((before + dindices) * 4) % 8 != 0;
  /* depth limit: the level count when unset or larger (GeoManager.cpp:220-221); deeper
     levels cache no matrix (NavIndexTable.cpp:18), the counting pass sizes the pad anyway */
  int levels          = g->max_depth + 1;
  int limit           = (g->cache_depth == 0 || g->cache_depth > levels) ? levels : g->cache_depth;
  int cache           = !(limit > 0 && level > limit);
  size_t cur_size     = (dindices + (size_t)pad) * 4 + (cache ? 12 * 8 : 0);
  unsigned char *bytes;
  or_xf mat;
  int i;
  double *m;

  if (v->count) {
    v->table_bytes += cur_size;
    return 0;
  }
  v->tab[v->current] = mother;
  if (mother > 0) v->tab[mother + 3 + dind] = v->current;
  v->tab[v->current + 1] = (uint32_t)pv;
  bytes    = (unsigned char *)&v->tab[v->current + 2];
  bytes[0] = (unsigned char)level;
  bytes[1] = 0;
  memcpy(bytes + 2, &nd, 2);
  for (i = 0; i < nd; ++i) v->tab[v->current + 3 + i] = 0;
  v->current += dindices;
  if (!cache) return new_mother;

  /* NavStatePath::TopMatrix (NavStatePath.h:616-628): identity times levels 1..level */
  xf_identity(&mat);
  for (i = 1; i <= level; ++i) xf_multiply_from_right(&mat, &g->pv[v->path[i]].xf);
  bytes[1] = (unsigned char)(0x04 + 0x02 * (mat.has_trans ? 1 : 0) + (mat.has_rot ? 1 : 0));
  if (pad) v->current++;
  m = (double *)&v->tab[v->current];
  for (i = 0; i < 3; ++i) m[i] = mat.t[i];
  for (i = 0; i < 9; ++i) m[3 + i] = mat.r[i];
  v->current += 24;
  return new_mother;
}

/* NavIndexTable::visitAllPlacedVolumesNavIndex (NavIndexTable.h:150-165) */
static void nav_visit(const or_geom *g, nav_visitor *v, int pv, int level, uint32_t mother, int dind)
{
  const or_lv *lv;
  uint32_t nm;
  int i;
  v->path[level] = pv;
  nm             = nav_apply(g, v, level, mother, dind);
  lv             = &g->lv[g->pv[pv].lv];
  for (i = 0; i < lv->nd; ++i) nav_visit(g, v, lv->daughters[i], level + 1, nm, i);
}

static int depth_of(const or_geom *g, int pv, int level)
{
  const or_lv *lv = &g->lv[g->pv[pv].lv];
  int i, d = level;
  for (i = 0; i < lv->nd; ++i) {
    int dd = depth_of(g, lv->daughters[i], level + 1);
    if (dd > d) d = dd;
  }
  return d;
}

static int shape_nparams(int type, const double *p, int avail)
{
  switch (type) {
  case OR_BOX: return 3;
  case OR_TUBE: return 5;
  case OR_CONE: return 7;
  case OR_TRD: return 5;
  case OR_TRAP: return 11;
  case OR_SPHERE: return 6;
  case OR_ORB: return 1;
  case OR_CUTTUBE: return 11;
  case OR_TORUS: return 5;
  case OR_BOOLEAN: return 3; /* op, left operand placement, right operand placement */
  case OR_POLYCONE: { /* sphi, dphi, nz, z[nz], rmin[nz], rmax[nz] */
    int nz;
    if (avail < 3 || !(p[2] >= 2 && p[2] <= 4096)) return -1;
    nz = (int)p[2];
    if ((double)nz != p[2]) return -1;
    return 3 + 3 * nz;
  }
  case OR_POLYHEDRON: { /* sphi, dphi, sides, nz, z[nz], rmin[nz], rmax[nz] */
    int nz;
    if (avail < 4 || !(p[3] >= 2 && p[3] <= 4096) || !(p[2] >= 1 && p[2] <= 4096)) return -1;
    nz = (int)p[3];
    if ((double)nz != p[3] || (double)(int)p[2] != p[2]) return -1;
    return 4 + 3 * nz;
  }
  default: (void)p; (void)avail; return -1;
  }
}

/* Boolean solids: each operand placement (pv_mother OR_BOOLEAN_OPERAND, anywhere in the
 * placement list) is used by exactly one boolean (UnplacedBooleanVolume.h:59 holds its own
 * placed operands); an operand's logical volume precedes its boolean, has no daughters and is
 * a primitive or a boolean of primitives.  Links each boolean to its operands and computes its
 * extent. */
static int link_booleans(or_geom *g, const int *pv_mother, char *err, int errlen)
{
  int i, used = 0, n_operands = 0, rc = 0;
  char *taken = (char *)calloc((size_t)g->n_pv + 1, 1);
  if (!taken) {
    set_err(err, errlen, "out of host memory");
    return -1;
  }
  for (i = 0; i < g->n_pv; ++i)
    if (pv_mother[i] == OR_BOOLEAN_OPERAND) ++n_operands;
  for (i = 0; i < g->n_lv; ++i) {
    or_boolean *b = &g->lv[i].s.boo;
    int k;
    if (g->lv[i].type != OR_BOOLEAN) continue;
    for (k = 0; k < 2; ++k) {
      const int pv = k == 0 ? b->left_pv : b->right_pv;
      const or_lv *o;
      if (pv < 0 || pv >= g->n_pv || pv_mother[pv] != OR_BOOLEAN_OPERAND || taken[pv]++) {
        set_err(err, errlen, "a boolean operand must be a placement with the operand mother, used once");
        rc = -1;
        goto done;
      }
      ++used;
      if (g->pv[pv].lv >= i) {
        set_err(err, errlen, "a boolean operand's logical volume must precede the boolean");
        rc = -1;
        goto done;
      }
      o = &g->lv[g->pv[pv].lv];
      if (o->nd != 0 || (o->type == OR_BOOLEAN && (o->s.boo.left->type == OR_BOOLEAN ||
                                                   o->s.boo.right->type == OR_BOOLEAN))) {
        set_err(err, errlen, "a boolean operand must have no daughters and be at most a boolean of primitives");
        rc = -1;
        goto done;
      }
      if (k == 0) {
        b->left = o;
        b->lxf  = g->pv[pv].xf;
      } else {
        b->right = o;
        b->rxf   = g->pv[pv].xf;
      }
    }
    shape_extent(&g->lv[i], &g->lv[i].bbox_min, &g->lv[i].bbox_max);
  }
  if (used != n_operands) {
    set_err(err, errlen, "a boolean operand placement is not used by exactly one boolean");
    rc = -1;
  }
done:
  free(taken);
  return rc;
}

or_geom *or_geom_create(int n_lv, const int *lv_shape, const int *lv_param_off, const double *params, int n_params,
                        int n_pv, const int *pv_lv, const int *pv_mother, const double *pv_trans, int world_pv,
                        char *err, int errlen)
{
  return or_geom_create_ex(n_lv, lv_shape, lv_param_off, params, n_params, n_pv, pv_lv, pv_mother, pv_trans,
                           world_pv, 0, err, errlen);
}

or_geom *or_geom_create_ex(int n_lv, const int *lv_shape, const int *lv_param_off, const double *params,
                           int n_params, int n_pv, const int *pv_lv, const int *pv_mother, const double *pv_trans,
                           int world_pv, int cache_depth, char *err, int errlen)
{
  or_geom *g;
  int i, *count;
  nav_visitor nv;

  if (n_lv <= 0 || n_pv <= 0 || world_pv < 0 || world_pv >= n_pv) {
    set_err(err, errlen, "empty geometry or bad world index");
    return NULL;
  }
  g        = (or_geom *)calloc(1, sizeof(or_geom));
  g->n_lv  = n_lv;
  g->n_pv  = n_pv;
  g->world_pv = world_pv;
  g->cache_depth = cache_depth < 0 ? 0 : cache_depth;
  g->lv    = (or_lv *)calloc((size_t)n_lv, sizeof(or_lv));
  g->pv    = (or_pv *)calloc((size_t)n_pv, sizeof(or_pv));
  for (i = 0; i < n_lv; ++i) {
    int np;
    g->lv[i].type      = lv_shape[i];
    g->lv[i].param_off = lv_param_off[i];
    np                 = shape_nparams(lv_shape[i], params + lv_param_off[i], n_params - lv_param_off[i]);
    if (np < 0 || lv_param_off[i] < 0 || lv_param_off[i] + np > n_params) {
      set_err(err, errlen, "unsupported shape type or parameters out of range");
      or_geom_free(g);
      return NULL;
    }
    if (shape_init(&g->lv[i], params + lv_param_off[i], n_params - lv_param_off[i], err, errlen)) {
      or_geom_free(g);
      return NULL;
    }
    if (lv_shape[i] != OR_BOOLEAN) /* ComputeBBox at construction; booleans once linked */
      shape_extent(&g->lv[i], &g->lv[i].bbox_min, &g->lv[i].bbox_max);
  }
  count = (int *)calloc((size_t)n_lv, sizeof(int));
  for (i = 0; i < n_pv; ++i) {
    if (pv_lv[i] < 0 || pv_lv[i] >= n_lv || pv_mother[i] < OR_BOOLEAN_OPERAND || pv_mother[i] >= n_lv) {
      set_err(err, errlen, "placed volume refers to an unknown logical volume");
      free(count);
      or_geom_free(g);
      return NULL;
    }
    g->pv[i].lv        = pv_lv[i];
    g->pv[i].mother_lv = pv_mother[i];
    xf_from12(&g->pv[i].xf, pv_trans + 12 * i);
    if (pv_mother[i] >= 0) g->lv[pv_mother[i]].nd++;
  }
  if (pv_mother[world_pv] != -1) {
    set_err(err, errlen, "world placement must have no mother");
    free(count);
    or_geom_free(g);
    return NULL;
  }
  if (link_booleans(g, pv_mother, err, errlen)) {
    free(count);
    or_geom_free(g);
    return NULL;
  }
  for (i = 0; i < n_lv; ++i)
    if (g->lv[i].nd) g->lv[i].daughters = (int *)malloc(sizeof(int) * (size_t)g->lv[i].nd);
  /* LogicalVolume::PlaceDaughter (source/LogicalVolume.cpp:142-148): child id = position */
  for (i = 0; i < n_pv; ++i) {
    int m = pv_mother[i];
    if (m < 0) continue;
    g->pv[i].child_id             = count[m];
    g->lv[m].daughters[count[m]++] = i;
  }
  free(count);

  g->max_depth = depth_of(g, world_pv, 0);
  if (g->max_depth > 30) {
    set_err(err, errlen, "geometry deeper than 30 levels");
    or_geom_free(g);
    return NULL;
  }

  /* ABBoxes + BVH per logical volume with daughters (BVHManager::Init, source/BVHManager.cpp:24-30) */
  for (i = 0; i < n_lv; ++i) {
    or_lv *lv = &g->lv[i];
    int k;
    if (!lv->nd) continue;
    lv->aabbs = (or_aabb *)malloc(sizeof(or_aabb) * (size_t)lv->nd);
    for (k = 0; k < lv->nd; ++k) compute_abbox(g, lv->daughters[k], &lv->aabbs[k]);
    if (bvh_build(g, i)) {
      set_err(err, errlen, "BVH build failed");
      or_geom_free(g);
      return NULL;
    }
  }

  /* two-pass navigation index table (NavIndexTable.h:114-132) */
  memset(&nv, 0, sizeof(nv));
  nv.count       = 1;
  nv.table_bytes = 4;
  nv.current     = 1;
  nav_visit(g, &nv, world_pv, 0, 0, 0);
  g->navind_words = nv.table_bytes / 4 + 1;
  g->navind       = (uint32_t *)calloc(g->navind_words + 1, 4);
  nv.count        = 0;
  nv.tab          = g->navind;
  nv.current      = 1;
  nav_visit(g, &nv, world_pv, 0, 0, 0);
  return g;
}

void or_geom_free(or_geom *g)
{
  int i;
  if (!g) return;
  if (g->lv) {
    for (i = 0; i < g->n_lv; ++i) {
      free(g->lv[i].daughters);
      free(g->lv[i].prim_id);
      free(g->lv[i].offset);
      free(g->lv[i].nchild);
      free(g->lv[i].nodes);
      free(g->lv[i].aabbs);
      if (g->lv[i].type == OR_POLYHEDRON) polyhedron_free(&g->lv[i].s.phd);
      if (g->lv[i].type == OR_POLYCONE) {
        free(g->lv[i].s.pcon.zs);
        free(g->lv[i].s.pcon.shift);
        free(g->lv[i].s.pcon.sec);
      }
    }
  }
  free(g->lv);
  free(g->pv);
  free(g->navind);
  free(g);
}

const uint32_t *or_geom_navindex(const or_geom *g, size_t *n_words)
{
  *n_words = g->navind_words;
  return g->navind;
}

int or_geom_bvh_info(const or_geom *g, int lv, int *depth, int *n_nodes, int *n_prims)
{
  if (lv < 0 || lv >= g->n_lv || !g->lv[lv].nd) return -1;
  *depth   = g->lv[lv].bvh_depth;
  *n_nodes = g->lv[lv].bvh_nodes;
  *n_prims = g->lv[lv].nd;
  return 0;
}

int or_geom_bvh_arrays(const or_geom *g, int lv, int *prim_id, int *offset, int *nchild, double *nodes_minmax,
                       double *prims_minmax)
{
  const or_lv *l;
  int i;
  if (lv < 0 || lv >= g->n_lv || !g->lv[lv].nd) return -1;
  l = &g->lv[lv];
  memcpy(prim_id, l->prim_id, sizeof(int) * (size_t)l->nd);
  memcpy(offset, l->offset, sizeof(int) * (size_t)l->bvh_nodes);
  memcpy(nchild, l->nchild, sizeof(int) * (size_t)l->bvh_nodes);
  for (i = 0; i < l->bvh_nodes; ++i) memcpy(nodes_minmax + 6 * i, &l->nodes[i], 6 * sizeof(double));
  for (i = 0; i < l->nd; ++i) memcpy(prims_minmax + 6 * i, &l->aabbs[i], 6 * sizeof(double));
  return 0;
}
