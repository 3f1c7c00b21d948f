/*
 * or_bvh.c -- oracle (test infrastructure): BVH construction with the
 * surface-area heuristic, restating source/BVH.cpp:48-87, 211-329, 359-385.
 *
 * std::sort is replaced by a heap-free merge sort on a strict total order
 * (the reference's less3D comparator makes every distinct key strictly
 * ordered, so any correct sort gives the same permutation); std::partition is
 * restated as libstdc++'s bidirectional-iterator partition, whose element
 * order within each half is what the reference's leaves end up holding.
 */
#include "or_internal.h"

/* AABB::SurfaceArea (AABB.h:51-56) */
static double aabb_area(const or_aabb *b)
{
  v3 e = v3_sub(b->mx, b->mn);
  return 2. * (e.x * e.y + e.y * e.z + e.z * e.x);
}

/* AABB::Union (AABB.h:212-219) */
static or_aabb aabb_union(const or_aabb *a, const or_aabb *b)
{
  or_aabb r;
  r.mn = v3_make(or_min(a->mn.x, b->mn.x), or_min(a->mn.y, b->mn.y), or_min(a->mn.z, b->mn.z));
  r.mx = v3_make(or_max(a->mx.x, b->mx.x), or_max(a->mx.y, b->mx.y), or_max(a->mx.z, b->mx.z));
  return r;
}

static double comp(v3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

/* sort key of the SAH sorter (BVH.cpp:284-291): centroid + 0.01 * (centroid - min) */
static v3 sah_key(const or_aabb *b)
{
  v3 c = v3_scale(0.5, v3_add(b->mx, b->mn));
  return v3_add(c, v3_scale(0.01, v3_sub(c, b->mn)));
}

/* less3D (BVH.cpp:217-225) */
static int less3d(v3 l, v3 r, int ax)
{
  int a1 = (ax + 1) % 3, a2 = (ax + 2) % 3;
  return comp(l, ax) < comp(r, ax) ||
         (comp(l, ax) == comp(r, ax) && (comp(l, a1) < comp(r, a1) || (comp(l, a1) == comp(r, a1) && comp(l, a2) < comp(r, a2))));
}

typedef struct {
  const or_aabb *boxes;
  int axis;
} sorter_ctx;

static int sorter_less(const sorter_ctx *s, int a, int b)
{
  return less3d(sah_key(&s->boxes[a]), sah_key(&s->boxes[b]), s->axis);
}

static void merge_sort(const sorter_ctx *s, int *a, int *tmp, long n)
{
  long mid, i, j, k;
  if (n < 2) return;
  mid = n / 2;
  merge_sort(s, a, tmp, mid);
  merge_sort(s, a + mid, tmp, n - mid);
  i = 0;
  j = mid;
  k = 0;
  while (i < mid && j < n) tmp[k++] = sorter_less(s, a[j], a[i]) ? a[j++] : a[i++];
  while (i < mid) tmp[k++] = a[i++];
  while (j < n) tmp[k++] = a[j++];
  memcpy(a, tmp, sizeof(int) * (size_t)n);
}

/* libstdc++ std::__partition for bidirectional iterators; pred(x) = sorter(x, pivot) */
static int *bidir_partition(const sorter_ctx *s, int *first, int *last, int pivot)
{
  for (;;) {
    for (;;) {
      if (first == last) return first;
      if (sorter_less(s, *first, pivot))
        ++first;
      else
        break;
    }
    --last;
    for (;;) {
      if (first == last) return first;
      if (!sorter_less(s, *last, pivot))
        --last;
      else
        break;
    }
    { int t = *first; *first = *last; *last = t; }
    ++first;
  }
}

/* surfaceAreaHeuristic (BVH.cpp:275-329) with sweepSurfaceArea (BVH.cpp:242-260) */
static int *sah_split(const or_aabb *boxes, int *begin, int *end)
{
  long nObj = end - begin, k;
  int bestSplitAxis = -1, bestSplitObject = -1, axis;
  double bestMetric = (double)nObj;
  double *first  = (double *)malloc(sizeof(double) * (size_t)nObj);
  double *second = (double *)malloc(sizeof(double) * (size_t)nObj);
  int *tmp       = (int *)malloc(sizeof(int) * (size_t)nObj);
  sorter_ctx s;
  s.boxes = boxes;

  for (axis = 0; axis <= 2; ++axis) {
    or_aabb box, box2;
    double tot;
    s.axis = axis;
    merge_sort(&s, begin, tmp, nObj);
    for (k = 0; k < nObj; ++k) first[k] = second[k] = 0.;
    box = boxes[begin[0]];
    for (k = 1; k < nObj; ++k) {
      first[k] = aabb_area(&box);
      box      = aabb_union(&box, &boxes[begin[k]]);
    }
    box2 = boxes[begin[nObj - 1]];
    for (k = nObj - 1; k >= 0; --k) {
      box2      = aabb_union(&box2, &boxes[begin[k]]);
      second[k] = aabb_area(&box2);
    }
    tot = second[0];
    for (k = 0; k < nObj; ++k) {
      const double left  = first[k] / tot;
      const double right = second[k] / tot;
      long bal           = nObj / 2 - k / nObj; /* integer arithmetic, as in the reference */
      const double metric = left * (double)k + right * (double)(nObj - k) + 0.1 * (double)(bal < 0 ? -bal : bal);
      if (metric < bestMetric) {
        bestMetric      = metric;
        bestSplitAxis   = axis;
        bestSplitObject = begin[k];
      }
    }
  }
  free(first);
  free(second);
  free(tmp);
  if (bestSplitAxis == -1) return end;
  s.axis = bestSplitAxis;
  return bidir_partition(&s, begin, end, bestSplitObject);
}

/* BVH::ComputeNodes (BVH.cpp:359-385) */
static void compute_nodes(or_lv *lv, unsigned id, int *first, int *last, unsigned nodes)
{
  int *it, *pivot;
  if (id >= nodes) return;
  lv->nchild[id] = (int)(last - first);
  lv->offset[id] = (int)(first - lv->prim_id);
  if (first == last) return;
  lv->nodes[id] = lv->aabbs[*first];
  for (it = first + 1; it != last; ++it) lv->nodes[id] = aabb_union(&lv->nodes[id], &lv->aabbs[*it]);
  if (first + 1 == last) return;
  pivot = sah_split(lv->aabbs, first, last);
  compute_nodes(lv, 2 * id + 1, first, pivot, nodes);
  compute_nodes(lv, 2 * id + 2, pivot, last, nodes);
}

/* BVH::BVH (BVH.cpp:48-87) */
int bvh_build(or_geom *g, int lvi)
{
  or_lv *lv = &g->lv[lvi];
  int n = lv->nd, i, half = n / 2;
  unsigned nodes, id;
  if (n <= 0) return -1;
  lv->prim_id = (int *)malloc(sizeof(int) * (size_t)n);
  for (i = 0; i < n; ++i) lv->prim_id[i] = i;
  lv->bvh_depth = half > 0 ? (int)log2((double)half) : 0;
  if (lv->bvh_depth < 0) lv->bvh_depth = 0;
  if (lv->bvh_depth > 32) lv->bvh_depth = 32;
  nodes         = (2u << lv->bvh_depth) - 1;
  lv->bvh_nodes = (int)nodes;
  lv->nchild    = (int *)calloc(nodes, sizeof(int));
  lv->offset    = (int *)malloc(sizeof(int) * nodes);
  lv->nodes     = (or_aabb *)calloc(nodes, sizeof(or_aabb)); /* default AABB: zero corners */
  for (id = 0; id < nodes; ++id) lv->offset[id] = -1;
  compute_nodes(lv, 0, lv->prim_id, lv->prim_id + n, nodes);
  for (id = 0; id < nodes / 2; ++id)
    if (lv->nchild[id] > 8 && (lv->nchild[id] == lv->nchild[2 * id + 1] + lv->nchild[2 * id + 2])) lv->nchild[id] = -1;
  return 0;
}
