/*
 * ORACLE - test infrastructure only.  Restatement of the reference's
 * geometry path: Tri::hit (src/tfg-pathtracer/Tri.hpp:38-160), the Ray
 * constructor (Ray.hpp:14-18), the fixed-depth binned-SAH BVH build
 * (BVH.hpp:187-211, 291-330, 373-460, 492-578) and its iterative traversal
 * (BVH.hpp:69-101, 120-185).
 */
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include "orc.h"
#ifdef _OPENMP
#include <omp.h>
#endif

/* Ray.hpp:14-18 */
orc_ray orc_make_ray(v3 o, v3 d) {
  orc_ray r;
  r.origin = o;
  r.direction = vnormalize(d);
  return r;
}

/* Tri.hpp:34-36 */
static inline v3 project_on_plane(v3 position, v3 origin, v3 normal) {
  return vsub(position, vscale(normal, vdot(vsub(position, origin), normal)));
}

/* Tri.hpp:38-160 with SMOOTH_SHADING (Definitions.h:3).  The epsilon is the
 * float nearest 1e-7; 1.0/det is a double division rounded to float. */
int orc_tri_hit(const orc_tri* t, const orc_ray* ray, orc_hit* hit) {
  const float EPSILON = (float)0.0000001;
  v3 edge1 = vsub(t->v[1], t->v[0]);
  v3 edge2 = vsub(t->v[2], t->v[0]);
  v3 pvec = vcross(ray->direction, edge2);
  float det = vdot(edge1, pvec);
  float inv_det = (float)(1.0 / (double)det);
  if (det > -EPSILON && det < EPSILON) return 0;
  v3 tvec = vsub(ray->origin, t->v[0]);
  float u = vdot(tvec, pvec) * inv_det;
  if (u < 0.0 || u > 1.0) return 0;
  v3 qvec = vcross(tvec, edge1);
  float v = vdot(ray->direction, qvec) * inv_det;
  if (v < 0.0 || (u + v) > 1.0) return 0;
  float tt = vdot(edge2, qvec) * inv_det;
  if (tt < 0) return 0;

  v3 tUV = vadd(vadd(t->uv[0], vscale(vsub(t->uv[1], t->uv[0]), u)), vscale(vsub(t->uv[2], t->uv[0]), v));
  v3 geom = vadd(ray->origin, vscale(ray->direction, tt));
  v3 sn = vadd(vadd(t->n[0], vscale(vsub(t->n[1], t->n[0]), u)), vscale(vsub(t->n[2], t->n[0]), v));
  v3 st = vadd(vadd(t->tg[0], vscale(vsub(t->tg[1], t->tg[0]), u)), vscale(vsub(t->tg[2], t->tg[0]), v));
  v3 p0 = project_on_plane(geom, t->v[0], t->n[0]);
  v3 p1 = project_on_plane(geom, t->v[1], t->n[1]);
  v3 p2 = project_on_plane(geom, t->v[2], t->n[2]);
  v3 sp = vadd(vadd(p0, vscale(vsub(p1, p0), u)), vscale(vsub(p2, p0), v));
  int convex = vdot(vsub(sp, geom), sn) > 0.0f;
  hit->tangent = st;
  hit->position = convex ? sp : geom;
  hit->normal = sn;
  hit->bitangent = vscale(vcross(hit->normal, hit->tangent), t->tsign);
  hit->valid = 1;
  hit->tu = tUV.x;
  hit->tv = tUV.y;
  hit->id = t->id;
  return 1;
}

/* ------------------------------------------------------------------ build */

typedef struct {
  const orc_tri* tris;
  orc_node* nodes;
  int32_t* tri_indices;
  int32_t nodeIdx, triIdx;
  int32_t* tmp;
} build_ctx;

/* BVH.hpp:529-538 */
static void tri_bounds(const orc_tri* t, v3* b1, v3* b2) {
  b1->x = minf_(t->v[0].x, minf_(t->v[1].x, t->v[2].x));
  b1->y = minf_(t->v[0].y, minf_(t->v[1].y, t->v[2].y));
  b1->z = minf_(t->v[0].z, minf_(t->v[1].z, t->v[2].z));
  b2->x = maxf_(t->v[0].x, maxf_(t->v[1].x, t->v[2].x));
  b2->y = maxf_(t->v[0].y, maxf_(t->v[1].y, t->v[2].y));
  b2->z = maxf_(t->v[0].z, maxf_(t->v[1].z, t->v[2].z));
}

/* BVH.hpp:540-578: leaves b1/b2 untouched for an empty list. */
static void list_bounds(const build_ctx* c, const int32_t* idx, int64_t n, v3* b1, v3* b2) {
  if (n <= 0) return;
  *b1 = c->tris[idx[0]].v[0];
  *b2 = c->tris[idx[0]].v[0];
  for (int64_t i = 0; i < n; i++) {
    const orc_tri* t = &c->tris[idx[i]];
    for (int k = 0; k < 3; k++) {
      b1->x = minf_(t->v[k].x, b1->x);
      b1->y = minf_(t->v[k].y, b1->y);
      b1->z = minf_(t->v[k].z, b1->z);
    }
    for (int k = 0; k < 3; k++) {
      b2->x = maxf_(t->v[k].x, b2->x);
      b2->y = maxf_(t->v[k].y, b2->y);
      b2->z = maxf_(t->v[k].z, b2->z);
    }
  }
}

/* BVH.hpp:519-527 */
static float bounds_area(v3 b1, v3 b2) {
  float x = b2.x - b1.x, y = b2.y - b1.y, z = b2.z - b1.z;
  return 2.0f * (x * y + x * z + y * z);
}

/* BVH.hpp:492-517: a zero-area box counts as empty. */
static void bounds_union(v3 b1, v3 b2, v3 b3, v3 b4, v3* b5, v3* b6) {
  if (bounds_area(b1, b2) <= 0 || bounds_area(b3, b4) <= 0) {
    if (bounds_area(b1, b2) <= 0) { *b5 = b3; *b6 = b4; }
    if (bounds_area(b3, b4) <= 0) { *b5 = b1; *b6 = b2; }
  } else {
    b5->x = minf_(b1.x, minf_(b2.x, minf_(b3.x, b4.x)));
    b5->y = minf_(b1.y, minf_(b2.y, minf_(b3.y, b4.y)));
    b5->z = minf_(b1.z, minf_(b2.z, minf_(b3.z, b4.z)));
    b6->x = maxf_(b1.x, maxf_(b2.x, maxf_(b3.x, b4.x)));
    b6->y = maxf_(b1.y, maxf_(b2.y, maxf_(b3.y, b4.y)));
    b6->z = maxf_(b1.z, maxf_(b2.z, maxf_(b3.z, b4.z)));
  }
}

/* Tri.hpp:27-32 */
static v3 centroid(const orc_tri* t) {
  return vdivs(V3(t->v[0].x + t->v[1].x + t->v[2].x, t->v[0].y + t->v[1].y + t->v[2].y,
                  t->v[0].z + t->v[1].z + t->v[2].z), 3.0f);
}

/* BVH.hpp:373-460.  Stable partition of idx[0..n) into [left | right];
 * returns the left count.  The final partition has no guard for a zero
 * extent on the chosen axis: the bin is then NaN/inf converted to int with
 * host semantics (INT_MIN), which sends everything left. */
static int64_t divide_sah(build_ctx* c, int32_t* idx, int64_t n) {
  if (n <= 0) return 0;
  v3 tb1 = V1(0), tb2 = V1(0);
  int bestBin = 0, bestAxis = 0;
  float bestH = FLT_MAX;
  list_bounds(c, idx, n, &tb1, &tb2);
  for (int axis = 0; axis < 3; axis++) {
    v3 b1s[ORC_SAH_BINS], b2s[ORC_SAH_BINS];
    int count[ORC_SAH_BINS];
    for (int i = 0; i < ORC_SAH_BINS; i++) { count[i] = 0; b1s[i] = V1(0); b2s[i] = V1(0); }
    float lo = vcomp(tb1, axis), hi = vcomp(tb2, axis);
    for (int64_t i = 0; i < n; i++) {
      int bin = 0;
      v3 b1, b2;
      if (lo != hi) {
        float cc = vcomp(centroid(&c->tris[idx[i]]), axis);
        bin = f2i_host(mapf_(cc, lo, hi, 0.0f, (float)(ORC_SAH_BINS - 1)));
      }
      count[bin]++;
      tri_bounds(&c->tris[idx[i]], &b1, &b2);
      bounds_union(b1s[bin], b2s[bin], b1, b2, &b1s[bin], &b2s[bin]);
    }
    for (int i = 0; i < ORC_SAH_BINS; i++) {
      int count1 = 0, count2 = 0;
      v3 b1 = V1(0), b2 = V1(0), b3 = V1(0), b4 = V1(0);
      for (int j = 0; j < i; j++) { count1 += count[j]; bounds_union(b1, b2, b1s[j], b2s[j], &b1, &b2); }
      for (int k = i; k < ORC_SAH_BINS; k++) { count2 += count[k]; bounds_union(b3, b4, b1s[k], b2s[k], &b3, &b4); }
      float h = bounds_area(b1, b2) * (float)count1 + bounds_area(b3, b4) * (float)count2;
      if (h < bestH) { bestH = h; bestBin = i; bestAxis = axis; }
    }
  }
  float lo = vcomp(tb1, bestAxis), hi = vcomp(tb2, bestAxis);
  int64_t nl = 0, nr = 0;
  int32_t* right = c->tmp;
  for (int64_t i = 0; i < n; i++) {
    float cc = vcomp(centroid(&c->tris[idx[i]]), bestAxis);
    int bin = f2i_host(mapf_(cc, lo, hi, 0.0f, (float)(ORC_SAH_BINS - 1)));
    if (bin < bestBin) idx[nl++] = idx[i];
    else right[nr++] = idx[i];
  }
  memcpy(idx + nl, right, (size_t)nr * sizeof(int32_t));
  return nl;
}

/* BVH.hpp:291-330: nodes are written in DFS pre-order; idx = own slot. */
static void build_aux(build_ctx* c, int depth, int32_t* idx, int64_t n) {
  v3 b1 = V1(0), b2 = V1(0);
  list_bounds(c, idx, n, &b1, &b2);
  orc_node* nd = &c->nodes[c->nodeIdx];
  nd->b1 = b1; nd->b2 = b2; nd->idx = c->nodeIdx; nd->depth = depth; nd->valid = 1;
  c->nodeIdx++;
  if (depth == ORC_BVH_DEPTH) {
    nd->from = c->triIdx;
    nd->to = c->triIdx + (int32_t)n;
    for (int64_t i = 0; i < n; i++) c->tri_indices[c->triIdx++] = idx[i];
  } else {
    nd->from = 0; nd->to = 0;
    int64_t nl = divide_sah(c, idx, n);
    build_aux(c, depth + 1, idx, nl);
    build_aux(c, depth + 1, idx + nl, n - nl);
  }
}

static void build_bvh(orc_scene* s) {
  int64_t nn = (int64_t)2 << ORC_BVH_DEPTH; /* BVH.hpp:62 */
  s->nodes = (orc_node*)calloc((size_t)nn, sizeof(orc_node));
  s->nnodes = nn;
  s->tri_indices = (int32_t*)malloc((size_t)(s->ntri > 0 ? s->ntri : 1) * sizeof(int32_t));
  int32_t* idx = (int32_t*)malloc((size_t)(s->ntri > 0 ? s->ntri : 1) * sizeof(int32_t));
  build_ctx c;
  c.tris = s->tris; c.nodes = s->nodes; c.tri_indices = s->tri_indices;
  c.nodeIdx = 0; c.triIdx = 0;
  c.tmp = (int32_t*)malloc((size_t)(s->ntri > 0 ? s->ntri : 1) * sizeof(int32_t));
  for (int64_t i = 0; i < s->ntri; i++) idx[i] = (int32_t)i;
  build_aux(&c, 0, idx, s->ntri);
  free(c.tmp);
  free(idx);
}

/* -------------------------------------------------------------- traverse */

/* BVH.hpp:69-101 */
static int ref_box(const orc_ray* r, v3 b1, v3 b2) {
  v3 df;
  df.x = 1.0f / r->direction.x;
  df.y = 1.0f / r->direction.y;
  df.z = 1.0f / r->direction.z;
  float t1 = (b1.x - r->origin.x) * df.x;
  float t2 = (b2.x - r->origin.x) * df.x;
  float t3 = (b1.y - r->origin.y) * df.y;
  float t4 = (b2.y - r->origin.y) * df.y;
  float t5 = (b1.z - r->origin.z) * df.z;
  float t6 = (b2.z - r->origin.z) * df.z;
  float tmin = maxf_(maxf_(minf_(t1, t2), minf_(t3, t4)), minf_(t5, t6));
  float tmax = minf_(minf_(maxf_(t1, t2), maxf_(t3, t4)), maxf_(t5, t6));
  if (tmax < 0) return 0;
  if (tmin > tmax) return 0;
  return 1;
}

/* BVH.hpp:159-175: first valid hit, then strictly smaller distance. */
static void intersect_node(const orc_scene* s, const orc_ray* r, const orc_node* nd, orc_hit* nearest) {
  for (int32_t i = nd->from; i < nd->to; i++) {
    orc_hit h;
    if (orc_tri_hit(&s->tris[s->tri_indices[i]], r, &h)) {
      if (!nearest->valid) *nearest = h;
      else if (vlen(vsub(h.position, r->origin)) < vlen(vsub(nearest->position, r->origin))) *nearest = h;
    }
  }
}

static orc_node child_left(const orc_scene* s, int32_t idx, int32_t depth) {
  orc_node n;
  if (depth == ORC_BVH_DEPTH) { memset(&n, 0, sizeof n); return n; }
  return s->nodes[idx + 1];
}
static orc_node child_right(const orc_scene* s, int32_t idx, int32_t depth) {
  orc_node n;
  if (depth == ORC_BVH_DEPTH) { memset(&n, 0, sizeof n); return n; }
  return s->nodes[idx + (2 << (ORC_BVH_DEPTH - depth - 1))];
}

/* BVH.hpp:120-157: both children tested per pop; leaves are intersected from
 * their depth-17 parent, right leaf first; left is descended, right pushed. */
void orc_transverse(const orc_scene* s, orc_ray r, orc_hit* nearest) {
  orc_node stack[64];
  int sp = 0;
  memset(&stack[0], 0, sizeof(orc_node));
  stack[sp++].valid = 0;
  orc_node node = s->nodes[0];
  do {
    orc_node l = child_left(s, node.idx, node.depth);
    orc_node rr = child_right(s, node.idx, node.depth);
    int lo = ref_box(&r, l.b1, l.b2);
    int ro = ref_box(&r, rr.b1, rr.b2);
    if (node.depth == ORC_BVH_DEPTH - 1 && ro) intersect_node(s, &r, &rr, nearest);
    if (node.depth == ORC_BVH_DEPTH - 1 && lo) intersect_node(s, &r, &l, nearest);
    int tl = lo && node.depth != ORC_BVH_DEPTH - 1;
    int tr = ro && node.depth != ORC_BVH_DEPTH - 1;
    if (!tl && !tr) {
      node = stack[--sp];
    } else {
      node = tl ? l : rr;
      if (tl && tr) stack[sp++] = rr;
    }
  } while (node.valid);
}

/* Exhaustive closest hit in triangle index order (tie: first index wins, or
 * the lowest tie key in key mode).  Used to classify traversal mismatches. */
static void brute_closest(const orc_scene* s, const orc_ray* r, int use_key, orc_hit* nearest) {
  float best = 0;
  uint32_t bestk = 0;
  for (int64_t i = 0; i < s->ntri; i++) {
    orc_hit h;
    if (!orc_tri_hit(&s->tris[i], r, &h)) continue;
    float d = vlen(vsub(h.position, r->origin));
    uint32_t k = s->tie_key ? s->tie_key[i] : (uint32_t)i;
    if (!nearest->valid || d < best || (use_key && d == best && k < bestk)) {
      *nearest = h; best = d; bestk = k;
    }
  }
}

void orc_trace(const orc_scene* s, const float* rays, int64_t n, int32_t mode, int32_t normalize,
               int32_t* tri, float* dist, float* uv, int32_t nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256)
#endif
  for (int64_t i = 0; i < n; i++) {
    const float* q = rays + 6 * i;
    orc_ray r;
    r.origin = V3(q[0], q[1], q[2]);
    r.direction = V3(q[3], q[4], q[5]);
    if (normalize) r = orc_make_ray(r.origin, r.direction);
    orc_hit h;
    memset(&h, 0, sizeof h);
    if (mode == 0) orc_transverse(s, r, &h);
    else brute_closest(s, &r, mode == 2, &h);
    tri[i] = h.valid ? h.id : -1;
    if (dist) dist[i] = h.valid ? vlen(vsub(h.position, r.origin)) : 0.0f;
    if (uv) {
      /* barycentrics are not part of Hit; report texture uv instead */
      uv[2 * i] = h.valid ? h.tu : 0.0f;
      uv[2 * i + 1] = h.valid ? h.tv : 0.0f;
    }
  }
}

/* ------------------------------------------------------------------ scene */

static v3 rd3(const float* p, int64_t i) { return V3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

orc_scene* orc_scene_new(const er_scene_desc* d) {
  orc_scene* s = (orc_scene*)calloc(1, sizeof(orc_scene));
  s->cam = d->camera;
  s->ntri = d->tri_count;
  s->tris = (orc_tri*)calloc((size_t)(d->tri_count > 0 ? d->tri_count : 1), sizeof(orc_tri));
  s->tri_mat = (int32_t*)calloc((size_t)(d->tri_count > 0 ? d->tri_count : 1), sizeof(int32_t));
  if (d->tie_key) {
    s->tie_key = (uint32_t*)malloc((size_t)d->tri_count * sizeof(uint32_t));
    memcpy(s->tie_key, d->tie_key, (size_t)d->tri_count * sizeof(uint32_t));
  }
  for (int64_t i = 0; i < d->tri_count; i++) {
    orc_tri* t = &s->tris[i];
    for (int k = 0; k < 3; k++) {
      t->v[k] = rd3(d->positions, 3 * i + k);
      t->n[k] = d->normals ? rd3(d->normals, 3 * i + k) : V1(0);
      t->tg[k] = d->tangents ? rd3(d->tangents, 3 * i + k) : V1(0);
      t->uv[k] = d->uvs ? V3(d->uvs[6 * i + 2 * k], d->uvs[6 * i + 2 * k + 1], 0.0f) : V1(0);
    }
    t->tsign = d->tangent_sign ? d->tangent_sign[i] : 1.0f;
    t->id = (int32_t)i;
    int32_t obj = d->tri_object ? d->tri_object[i] : 0;
    s->tri_mat[i] = (d->object_material && obj >= 0 && obj < d->object_count) ? d->object_material[obj] : 0;
  }
  s->nmat = d->material_count;
  s->mats = (er_material*)calloc((size_t)(d->material_count > 0 ? d->material_count : 1), sizeof(er_material));
  if (d->material_count > 0) memcpy(s->mats, d->materials, (size_t)d->material_count * sizeof(er_material));
  s->ntex = d->texture_count;
  s->texs = (orc_tex*)calloc((size_t)(d->texture_count > 0 ? d->texture_count : 1), sizeof(orc_tex));
  s->tex_store = (float**)calloc((size_t)(d->texture_count > 0 ? d->texture_count : 1), sizeof(float*));
  for (int i = 0; i < d->texture_count; i++) {
    const er_texture* t = &d->textures[i];
    size_t bytes = (size_t)t->width * (size_t)t->height * 3 * sizeof(float);
    s->tex_store[i] = (float*)malloc(bytes);
    memcpy(s->tex_store[i], t->data, bytes);
    s->texs[i].w = t->width; s->texs[i].h = t->height; s->texs[i].data = s->tex_store[i];
    s->texs[i].xTile = t->x_tile; s->texs[i].yTile = t->y_tile;
    s->texs[i].xOffset = t->x_offset; s->texs[i].yOffset = t->y_offset;
  }
  s->nlights = d->light_count;
  s->lights = (er_point_light*)calloc((size_t)(d->light_count > 0 ? d->light_count : 1), sizeof(er_point_light));
  if (d->light_count > 0) memcpy(s->lights, d->lights, (size_t)d->light_count * sizeof(er_point_light));
  {
    const er_texture* t = &d->env;
    size_t np = (size_t)t->width * (size_t)t->height;
    s->env_store = (float*)malloc(np * 3 * sizeof(float) + 4);
    if (np) memcpy(s->env_store, t->data, np * 3 * sizeof(float));
    s->env.w = t->width; s->env.h = t->height; s->env.data = s->env_store;
    s->env.xTile = t->x_tile; s->env.yTile = t->y_tile;
    s->env.xOffset = t->x_offset; s->env.yOffset = t->y_offset;
    s->cdf = (float*)malloc((np + 1) * sizeof(float));
    orc_hdri_cdf(&s->env, s->cdf, &s->radianceSum);
  }
  build_bvh(s);
  return s;
}

void orc_scene_free(orc_scene* s) {
  if (!s) return;
  free(s->tris); free(s->tri_mat); free(s->tie_key); free(s->nodes); free(s->tri_indices);
  free(s->mats);
  for (int i = 0; i < s->ntex; i++) free(s->tex_store[i]);
  free(s->tex_store); free(s->texs); free(s->lights); free(s->env_store); free(s->cdf);
  free(s);
}

int64_t orc_bvh_node_count(const orc_scene* s) { return s->nnodes; }

void orc_bvh_export(const orc_scene* s, float* boxes, int32_t* meta, int32_t* tri_indices) {
  for (int64_t i = 0; i < s->nnodes; i++) {
    const orc_node* n = &s->nodes[i];
    if (boxes) {
      boxes[6 * i + 0] = n->b1.x; boxes[6 * i + 1] = n->b1.y; boxes[6 * i + 2] = n->b1.z;
      boxes[6 * i + 3] = n->b2.x; boxes[6 * i + 4] = n->b2.y; boxes[6 * i + 5] = n->b2.z;
    }
    if (meta) {
      meta[5 * i + 0] = n->from; meta[5 * i + 1] = n->to; meta[5 * i + 2] = n->idx;
      meta[5 * i + 3] = n->depth; meta[5 * i + 4] = n->valid;
    }
  }
  if (tri_indices && s->ntri > 0) memcpy(tri_indices, s->tri_indices, (size_t)s->ntri * sizeof(int32_t));
}
