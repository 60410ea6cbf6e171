/*
 * ORACLE - test infrastructure only (the FP64 reference for image error).
 * Nothing in the product library includes, links or calls this code.
 *
 * The reference's per-sample estimator restated in double precision:
 * camera ray (kernel.cu:260-337), closest hit with the smooth-shading
 * position ranking (Tri.hpp:38-160), generateHitData (kernel.cu:54-119),
 * DisneySample / DisneyEval / DisneyPdf (Disney.hpp:41-253, Sampling.hpp:
 * 31-54), pointLight (kernel.cu:175-205), hdriLight (kernel.cu:210-258,
 * HDRI.hpp:130-162), the MIS mix of shade (kernel.cu:339-358), the path loop
 * (kernel.cu:404-443) and the per-sample clamp / NaN drop of the
 * accumulation (kernel.cu:445-449), averaged in double.
 *
 * It has its own BVH (binary, median split of centroids, built here in
 * double) and a closest-hit traversal pruned by the best shading distance:
 * a node is skipped when its entry distance minus the largest shading
 * offset of its triangles exceeds the best distance found.  Random numbers
 * are the same Philox stream as the FP32 oracle and the GPU.  The
 * environment texel is chosen by the reference search over the scene's
 * FP32 CDF with the FP32 uniform, so the sampled texel distribution is the
 * one every renderer of this estimator uses; everything after that choice
 * is double.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI64 3.14159265358979323846

typedef struct { double x, y, z; } d3;

static inline d3 D(double x, double y, double z) { d3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline d3 Df(v3 a) { return D(a.x, a.y, a.z); }
static inline d3 add(d3 a, d3 b) { return D(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline d3 sub(d3 a, d3 b) { return D(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline d3 mul(d3 a, d3 b) { return D(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline d3 scl(d3 a, double s) { return D(a.x * s, a.y * s, a.z * s); }
static inline d3 dvs(d3 a, double s) { return D(a.x / s, a.y / s, a.z / s); }
static inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline d3 cross(d3 a, d3 b) { return D(a.y * b.z - a.z * b.y, -(a.x * b.z - a.z * b.x), a.x * b.y - a.y * b.x); }
static inline double len(d3 a) { return sqrt(dot(a, a)); }
/* Vector3::normalized: the input unchanged when its length is 0 */
static inline d3 nrm(d3 a) {
  double l = len(a);
  return l == 0 ? a : dvs(a, l);
}
static inline double lerp(double a, double b, double c) { return a + c * (b - a); }
static inline d3 lerp3(d3 a, d3 b, double c) { return D(lerp(a.x, b.x, c), lerp(a.y, b.y, c), lerp(a.z, b.z, c)); }
static inline double clampd(double a, double b, double c) { return a < b ? b : a > c ? c : a; }
static inline double maxd(double a, double b) { return a > b ? a : b; }
static inline void limit_uv64(double* u, double* v) {
  *u += (double)(-(*u > 1) + -(*u < 0));
  *v += (double)(-(*v > 1) + -(*v < 0));
}
static inline int32_t d2i(double f) {
  if (f != f) return 0;
  if (f >= 2147483647.0) return INT_MAX;
  if (f <= -2147483648.0) return INT_MIN;
  return (int32_t)f;
}

typedef struct { d3 o, d; } ray64;
static ray64 make_ray(d3 o, d3 d) { ray64 r; r.o = o; r.d = nrm(d); return r; }

typedef struct {
  d3 position, normal, tangent, bitangent;
  int valid;
  int32_t id;
  double tu, tv;
} hit64;

/* ------------------------------------------------------------------- BVH */

typedef struct {
  double lo[3], hi[3];
  double delta;          /* largest shading offset of the triangles below */
  int32_t left, right;   /* children, -1 for a leaf */
  int32_t first, count;  /* leaf range in idx */
} bnode;

typedef struct orc64_scene {
  const orc_scene* s;
  bnode* nodes;
  int32_t nn, cap;
  int32_t* idx;
  double* tdelta;
  double* cent;
  double radiance_sum;   /* environment radiance sum in double */
} orc64_scene;

/* Tri.hpp:74-92: |shading position - geometric hit| <= max over vertices a
 * of |n_a| * max_b |(v_b - v_a).n_a| (the hit is a convex combination of
 * the vertices and each projection moves it along n_a). */
static double shading_bound(const orc_tri* t) {
  double m = 0;
  for (int a = 0; a < 3; a++) {
    d3 n = Df(t->n[a]);
    double mx = 0;
    for (int b = 0; b < 3; b++) mx = maxd(mx, fabs(dot(sub(Df(t->v[b]), Df(t->v[a])), n)));
    m = maxd(m, len(n) * mx);
  }
  return m * (1.0 + 1e-9);
}

static int32_t build(orc64_scene* S, int32_t b, int32_t e) {
  const orc_scene* s = S->s;
  if (S->nn == S->cap) {
    S->cap = S->cap ? 2 * S->cap : 1024;
    S->nodes = (bnode*)realloc(S->nodes, (size_t)S->cap * sizeof(bnode));
  }
  int32_t me = S->nn++;
  bnode nd;
  for (int k = 0; k < 3; k++) { nd.lo[k] = INFINITY; nd.hi[k] = -INFINITY; }
  nd.delta = 0;
  double clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int32_t i = b; i < e; i++) {
    const orc_tri* t = &s->tris[S->idx[i]];
    for (int v = 0; v < 3; v++) {
      double p[3] = {t->v[v].x, t->v[v].y, t->v[v].z};
      for (int k = 0; k < 3; k++) { nd.lo[k] = fmin(nd.lo[k], p[k]); nd.hi[k] = fmax(nd.hi[k], p[k]); }
    }
    for (int k = 0; k < 3; k++) {
      double c = S->cent[3 * (int64_t)S->idx[i] + k];
      clo[k] = fmin(clo[k], c);
      chi[k] = fmax(chi[k], c);
    }
    nd.delta = maxd(nd.delta, S->tdelta[S->idx[i]]);
  }
  nd.first = b;
  nd.count = e - b;
  nd.left = nd.right = -1;
  if (e - b > 4) {
    int ax = 0;
    for (int k = 1; k < 3; k++)
      if (chi[k] - clo[k] > chi[ax] - clo[ax]) ax = k;
    double mid = 0.5 * (clo[ax] + chi[ax]);
    int32_t i = b, j = e - 1;
    while (i <= j) {
      if (S->cent[3 * (int64_t)S->idx[i] + ax] < mid) i++;
      else { int32_t tmp = S->idx[i]; S->idx[i] = S->idx[j]; S->idx[j] = tmp; j--; }
    }
    int32_t m = i;
    if (m == b || m == e) m = b + (e - b) / 2;
    int32_t l = build(S, b, m);
    int32_t r = build(S, m, e);
    nd.left = l;
    nd.right = r;
  }
  S->nodes[me] = nd;
  return me;
}

orc64_scene* orc64_new(const orc_scene* s) {
  orc64_scene* S = (orc64_scene*)calloc(1, sizeof(orc64_scene));
  S->s = s;
  int64_t T = s->ntri;
  S->idx = (int32_t*)malloc((size_t)(T > 0 ? T : 1) * sizeof(int32_t));
  S->tdelta = (double*)malloc((size_t)(T > 0 ? T : 1) * sizeof(double));
  S->cent = (double*)malloc((size_t)(T > 0 ? 3 * T : 3) * sizeof(double));
  for (int64_t i = 0; i < T; i++) {
    const orc_tri* t = &s->tris[i];
    S->idx[i] = (int32_t)i;
    S->tdelta[i] = shading_bound(t);
    S->cent[3 * i] = ((double)t->v[0].x + t->v[1].x + t->v[2].x) / 3.0;
    S->cent[3 * i + 1] = ((double)t->v[0].y + t->v[1].y + t->v[2].y) / 3.0;
    S->cent[3 * i + 2] = ((double)t->v[0].z + t->v[1].z + t->v[2].z) / 3.0;
  }
  if (T > 0) build(S, 0, (int32_t)T);
  double sum = 0;
  const orc_tex* e = &s->env;
  for (int32_t j = 0; j < e->h; j++)
    for (int32_t i = 0; i < e->w; i++) {
      v3 c = orc_tex_coord(e, i, j);
      sum += ((double)c.x + c.y) + c.z;
    }
  S->radiance_sum = sum;
  return S;
}

void orc64_free(orc64_scene* S) {
  if (!S) return;
  free(S->nodes); free(S->idx); free(S->tdelta); free(S->cent);
  free(S);
}

/* Tri.hpp:38-160 in double (same epsilon on the determinant). */
static int tri_hit64(const orc_tri* t, const ray64* r, hit64* h, double* dist) {
  const double EPS = (double)(float)0.0000001;
  d3 v0 = Df(t->v[0]), v1 = Df(t->v[1]), v2 = Df(t->v[2]);
  d3 e1 = sub(v1, v0), e2 = sub(v2, v0);
  d3 pv = cross(r->d, e2);
  double det = dot(e1, pv);
  if (det > -EPS && det < EPS) return 0;
  double inv = 1.0 / det;
  d3 tv = sub(r->o, v0);
  double u = dot(tv, pv) * inv;
  if (u < 0.0 || u > 1.0) return 0;
  d3 qv = cross(tv, e1);
  double v = dot(r->d, qv) * inv;
  if (v < 0.0 || u + v > 1.0) return 0;
  double tt = dot(e2, qv) * inv;
  if (tt < 0) return 0;
  d3 geom = add(r->o, scl(r->d, tt));
  d3 n0 = Df(t->n[0]), n1 = Df(t->n[1]), n2 = Df(t->n[2]);
  d3 sn = add(add(n0, scl(sub(n1, n0), u)), scl(sub(n2, n0), v));
  d3 g0 = Df(t->tg[0]), g1 = Df(t->tg[1]), g2 = Df(t->tg[2]);
  d3 st = add(add(g0, scl(sub(g1, g0), u)), scl(sub(g2, g0), v));
  d3 p0 = sub(geom, scl(n0, dot(sub(geom, v0), n0)));
  d3 p1 = sub(geom, scl(n1, dot(sub(geom, v1), n1)));
  d3 p2 = sub(geom, scl(n2, dot(sub(geom, v2), n2)));
  d3 sp = add(add(p0, scl(sub(p1, p0), u)), scl(sub(p2, p0), v));
  int convex = dot(sub(sp, geom), sn) > 0.0;
  d3 uv0 = Df(t->uv[0]), uv1 = Df(t->uv[1]), uv2 = Df(t->uv[2]);
  d3 tuv = add(add(uv0, scl(sub(uv1, uv0), u)), scl(sub(uv2, uv0), v));
  h->position = convex ? sp : geom;
  h->normal = sn;
  h->tangent = st;
  h->bitangent = scl(cross(sn, st), t->tsign);
  h->valid = 1;
  h->id = t->id;
  h->tu = tuv.x;
  h->tv = tuv.y;
  *dist = len(sub(h->position, r->o));
  return 1;
}

static int box_enter(const bnode* n, const ray64* r, double* tmin) {
  double t0 = -INFINITY, t1 = INFINITY;
  const double o[3] = {r->o.x, r->o.y, r->o.z}, d[3] = {r->d.x, r->d.y, r->d.z};
  for (int k = 0; k < 3; k++) {
    if (d[k] == 0.0) {
      if (o[k] < n->lo[k] || o[k] > n->hi[k]) return 0;
      continue;
    }
    double a = (n->lo[k] - o[k]) / d[k], b = (n->hi[k] - o[k]) / d[k];
    if (a > b) { double tmp = a; a = b; b = tmp; }
    t0 = fmax(t0, a);
    t1 = fmin(t1, b);
  }
  /* widened by a relative margin: the box holds float vertices exactly */
  double m = 1e-9 * (fabs(t0) + fabs(t1) + 1.0);
  if (t1 + m < 0 || t0 > t1 + m) return 0;
  *tmin = t0;
  return 1;
}

/* closest hit by shading-position distance (kernel.cu:152-173) */
static hit64 closest(const orc64_scene* S, const ray64* r) {
  hit64 best;
  memset(&best, 0, sizeof best);
  double bd = INFINITY;
  if (S->nn == 0) return best;
  int32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const bnode* n = &S->nodes[stack[--sp]];
    double tmin;
    if (!box_enter(n, r, &tmin)) continue;
    if (tmin - n->delta > bd * (1.0 + 1e-12)) continue;
    if (n->left < 0) {
      for (int32_t i = n->first; i < n->first + n->count; i++) {
        hit64 h;
        double dd;
        if (tri_hit64(&S->s->tris[S->idx[i]], r, &h, &dd) && dd < bd) {
          bd = dd;
          best = h;
        }
      }
    } else if (sp + 2 <= 128) {
      stack[sp++] = n->right;
      stack[sp++] = n->left;
    }
  }
  return best;
}

/* ------------------------------------------------------------- shading */

/* Evaluation parameters of the detached estimator (as er_render_replay):
 * sampling uses the scene's materials and environment, BRDF values and
 * environment radiance these (NULL = the scene's). */
typedef struct {
  const float* mat; /* n_materials x 5: albedo rgb, roughness, metallic */
  const float* env; /* env w*h*3, storage order */
} eval64;

/* storage index of the texel orc_tex_coord reads (Texture.hpp:95-112) */
static int64_t tex_index64(const orc_tex* t, int32_t x, int32_t y) {
  x = f2i_dev(t->xTile * ((float)x + t->xOffset * (float)t->w)) % t->w;
  y = f2i_dev(t->yTile * ((float)y + t->yOffset * (float)t->h)) % t->h;
  if (x < 0) x += t->w;
  if (y < 0) y += t->h;
  return (int64_t)y * t->w + x;
}

static d3 env_value64(const orc_tex* t, const eval64* ev, double u, double v) {
  int32_t x = d2i(u * (double)t->w), y = d2i(v * (double)t->h);
  if (ev && ev->env) {
    const float* p = ev->env + 3 * tex_index64(t, x, y);
    return D(p[0], p[1], p[2]);
  }
  return Df(orc_tex_coord(t, x, y));
}

typedef struct {
  double metallic, roughness, clearcoatGloss, clearcoat, anisotropic, transmission, specular, specularTint,
      sheenTint, subsurface, sheen;
  d3 emission, albedo, normal;
} hd64;

static d3 tex_uv64(const orc_tex* t, double u, double v) {
  return Df(orc_tex_coord(t, d2i(u * (double)t->w), d2i(v * (double)t->h)));
}

static void spherical64(d3 p, double* u, double* v) {
  double theta = acos(-p.y);
  double phi = atan2(-p.z, p.x) + PI64;
  *u = phi / (2.0 * PI64);
  *v = theta / PI64;
  limit_uv64(u, v);
}

static d3 reverse_spherical64(double u, double v) {
  double phi = u * 2.0 * PI64, theta = v * PI64;
  double py = -cos(theta);
  double a = sqrt(1.0 - py * py);
  return D(a * cos(phi - PI64), py, a * -sin(phi - PI64));
}

static void hit_data64(const orc_scene* s, const er_material* m, const hit64* h, hd64* hd) {
  hd->albedo = m->albedo_tex < 0 ? D(m->albedo[0], m->albedo[1], m->albedo[2]) : tex_uv64(&s->texs[m->albedo_tex], h->tu, h->tv);
  hd->emission = m->emission_tex < 0 ? D(m->emission[0], m->emission[1], m->emission[2])
                                     : tex_uv64(&s->texs[m->emission_tex], h->tu, h->tv);
  double rough = m->roughness_tex < 0 ? m->roughness : tex_uv64(&s->texs[m->roughness_tex], h->tu, h->tv).x;
  double metal = m->metallic_tex < 0 ? m->metallic : tex_uv64(&s->texs[m->metallic_tex], h->tu, h->tv).x;
  if (m->normal_tex < 0) {
    hd->normal = h->normal;
  } else {
    d3 c = tex_uv64(&s->texs[m->normal_tex], h->tu, h->tv);
    d3 ln = sub(scl(c, 2.0), D(1, 1, 1));
    hd->normal = nrm(add(sub(scl(h->tangent, ln.x), scl(h->bitangent, ln.y)), scl(h->normal, ln.z)));
  }
  hd->roughness = pow(rough, 2.2);
  hd->metallic = pow(metal, 2.2);
  hd->clearcoatGloss = m->clearcoat_gloss;
  hd->clearcoat = m->clearcoat;
  hd->anisotropic = m->anisotropic;
  hd->transmission = m->transmission;
  hd->specular = m->specular;
  hd->specularTint = m->specular_tint;
  hd->sheenTint = m->sheen_tint;
  hd->subsurface = m->subsurface;
  hd->sheen = m->sheen;
}

/* the evaluation copy of a vertex's HitData */
static void hit_data_eval64(const er_material* m, int32_t mat_id, const eval64* ev, const hd64* hs, hd64* he) {
  *he = *hs;
  if (!ev || !ev->mat) return;
  const float* q = ev->mat + 5 * (int64_t)mat_id;
  if (m->albedo_tex < 0) he->albedo = D(q[0], q[1], q[2]);
  if (m->roughness_tex < 0) he->roughness = pow((double)q[3], 2.2);
  if (m->metallic_tex < 0) he->metallic = pow((double)q[4], 2.2);
}

static void basis64(d3 n, d3* t, d3* b) {
  *t = nrm(cross(D(0, 1, 0), n));
  *b = nrm(cross(n, *t));
}
static double schlick64(double u) {
  double m = clampd(1.0 - u, 0.0, 1.0), m2 = m * m;
  return m2 * m2 * m;
}
static double gtr1_64(double NDotH, double a) {
  if (a >= 1.0) return 1.0 / PI64;
  double a2 = a * a;
  double t = 1.0 + (a2 - 1.0) * NDotH * NDotH;
  return (a2 - 1.0) / (PI64 * log(a2) * t);
}
static double gtr2_aniso64(double NDotH, double HDotX, double HDotY, double ax, double ay) {
  double a = HDotX / ax, b = HDotY / ay, c = a * a + b * b + NDotH * NDotH;
  return 1.0 / (PI64 * ax * ay * c * c);
}
static double smith_ggx64(double NDotV, double alphaG) {
  double a = alphaG * alphaG, b = NDotV * NDotV;
  return 1.0 / (NDotV + sqrt(a + b - a * b));
}
static double smith_ggx_aniso64(double NDotV, double VDotX, double VDotY, double ax, double ay) {
  double a = VDotX * ax, b = VDotY * ay;
  return 1.0 / (NDotV + sqrt(a * a + b * b + NDotV * NDotV));
}

static double disney_pdf64(const ray64* r, const hd64* hd, d3 L) {
  d3 N = hd->normal, V = scl(r->d, -1.0);
  d3 H = nrm(add(L, V)), T, B;
  basis64(N, &T, &B);
  double NDotH = fabs(dot(N, H));
  if (dot(N, L) <= 0.0) return 1.0;
  double ccAlpha = lerp(0.1, 0.001, hd->clearcoatGloss);
  double diffuseRatio = 0.5 * (1.0 - hd->metallic), specularRatio = 1.0 - diffuseRatio;
  double aspect = sqrt(1.0 - hd->anisotropic * 0.9);
  double ax = maxd(0.001, hd->roughness / aspect), ay = maxd(0.001, hd->roughness * aspect);
  double pdfGTR2 = gtr2_aniso64(NDotH, dot(H, T), dot(H, B), ax, ay) * NDotH;
  double pdfGTR1 = gtr1_64(NDotH, ccAlpha) * NDotH;
  double ratio = 1.0 / (1.0 + hd->clearcoat);
  double pdfSpec = lerp(pdfGTR1, pdfGTR2, ratio) / (4.0 * fabs(dot(L, H)));
  double pdfDiff = fabs(dot(L, N)) * (1.0 / PI64);
  return diffuseRatio * pdfDiff + specularRatio * pdfSpec;
}

static d3 disney_sample64(const ray64* r, const hd64* hd, double r1, double r2, double r3) {
  d3 N = hd->normal, V = scl(r->d, -1.0), T, B;
  basis64(N, &T, &B);
  double diffuseRatio = 0.5 * (1.0 - hd->metallic);
  if (r3 < diffuseRatio) {
    double rr = sqrt(r1), phi = 2.0 * PI64 * r2;
    double hx = rr * cos(phi), hy = rr * sin(phi);
    double hz = sqrt(maxd(0.0, 1.0 - hx * hx - hy * hy));
    return add(add(scl(T, hx), scl(B, hy)), scl(N, hz));
  }
  double a = maxd(0.001, hd->roughness);
  double phi = r1 * PI64 * 2.0;
  double cosT = sqrt((1.0 - r2) / (1.0 + (a * a - 1.0) * r2));
  double sinT = clampd(sqrt(1.0 - cosT * cosT), 0.0, 1.0);
  d3 H = add(add(scl(T, sinT * cos(phi)), scl(B, sinT * sin(phi))), scl(N, cosT));
  d3 v = scl(V, -1.0);
  return sub(v, scl(H, 2.0 * dot(v, H)));
}

static d3 disney_eval64(const ray64* r, const hd64* hd, d3 L) {
  d3 V = scl(r->d, -1.0), T, B;
  basis64(hd->normal, &T, &B);
  if (!(hd->transmission < 1.0 && dot(hd->normal, L) > 0.0 && dot(hd->normal, V) > 0.0)) return D(0, 0, 0);
  d3 H = nrm(add(L, V));
  double NDotL = fabs(dot(hd->normal, L)), NDotV = fabs(dot(hd->normal, V));
  double NDotH = fabs(dot(hd->normal, H)), LDotH = fabs(dot(L, H));
  d3 Cdlin = hd->albedo;
  double Cdlum = 0.3 * Cdlin.x + 0.6 * Cdlin.y + 0.1 * Cdlin.z;
  d3 Ctint = Cdlum > 0.0 ? dvs(Cdlin, Cdlum) : D(1, 1, 1);
  d3 Cspec0 = lerp3(scl(lerp3(D(1, 1, 1), Ctint, hd->specularTint), hd->specular * 0.08), Cdlin, hd->metallic);
  d3 Csheen = lerp3(D(1, 1, 1), Ctint, hd->sheenTint);
  double FL = schlick64(NDotL), FV = schlick64(NDotV);
  double Fd90 = 0.5 + 2.0 * LDotH * LDotH * hd->roughness;
  double Fd = lerp(1.0, Fd90, FL) * lerp(1.0, Fd90, FV);
  double Fss90 = LDotH * LDotH * hd->roughness;
  double Fss = lerp(1.0, Fss90, FL) * lerp(1.0, Fss90, FV);
  double ss = 1.25 * (Fss * (1.0 / (NDotL + NDotV) - 0.5) + 0.5);
  double aspect = sqrt(1.0 - hd->anisotropic * 0.9);
  double ax = maxd(0.001, hd->roughness / aspect), ay = maxd(0.001, hd->roughness * aspect);
  double Ds = gtr2_aniso64(NDotH, dot(H, T), dot(H, B), ax, ay);
  double FH = schlick64(LDotH);
  d3 Fs = lerp3(Cspec0, D(1, 1, 1), FH);
  double Gs = smith_ggx_aniso64(NDotL, dot(L, T), dot(L, B), ax, ay) *
              smith_ggx_aniso64(NDotV, dot(V, T), dot(V, B), ax, ay);
  d3 Fsheen = scl(Csheen, FH * hd->sheen);
  double Dr = gtr1_64(NDotH, lerp(0.1, 0.001, hd->clearcoatGloss));
  double Fr = lerp(0.04, 1.0, FH);
  double Gr = smith_ggx64(NDotL, 0.25) * smith_ggx64(NDotV, 0.25);
  double kd = (1.0 / PI64) * lerp(Fd, ss, hd->subsurface);
  d3 diff = scl(add(scl(Cdlin, kd), Fsheen), 1.0 - hd->metallic);
  d3 spec = scl(scl(Fs, Gs), Ds);
  double cc = 0.25 * hd->clearcoat * Gr * Fr * Dr;
  return add(add(diff, spec), D(cc, cc, cc));
}

static ray64 camera64(const er_camera* c, int32_t x, int32_t y, const double* u) {
  double dx = c->position[0] + (double)x / c->x_res * c->sensor_width;
  double dy = c->position[1] + (double)y / c->y_res * c->sensor_height;
  double odx = -(double)c->sensor_width / 2.0 + dx, ody = -(double)c->sensor_height / 2.0 + dy;
  double rx = (1.0 / c->x_res) * (u[0] - 0.5) * c->sensor_width;
  double ry = (1.0 / c->y_res) * (u[1] - 0.5) * c->sensor_height;
  d3 SP = D(odx + rx, ody + ry, (double)c->position[2] + c->focal_length);
  double k = PI64 / 180.0;
  double ax = c->rotation[0] * k, ay = c->rotation[1] * k, az = c->rotation[2] * k;
  d3 pos = D(c->position[0], c->position[1], c->position[2]);
  d3 d = sub(SP, pos);
  d3 dX = D(d.x, d.y * cos(ax) - d.z * sin(ax), d.y * sin(ax) + d.z * cos(ax));
  d3 dY = D(dX.x * cos(ay) + dX.z * sin(ay), dX.y, dX.z * cos(ay) - dX.x * sin(ay));
  d3 dZ = D(dY.x * cos(az) - dY.y * sin(az), dY.x * sin(az) + dY.y * cos(az), dY.z);
  ray64 r = make_ray(pos, dZ);
  if (c->bokeh) {
    double diameter = (double)c->focal_length / c->aperture;
    double l = (double)c->focus_distance + c->focal_length;
    d3 focus = add(r.o, scl(r.d, l));
    double t = 2.0 * PI64 * u[2], s = u[3] + u[4];
    double rr = s > 1 ? 2 - s : s;
    d3 orig = add(pos, D(rr * cos(t) * diameter * 0.5, rr * sin(t) * diameter * 0.5, 0));
    r = make_ray(orig, sub(focus, orig));
  }
  return r;
}

/* kernel.cu:175-205 */
static d3 point_light64(const orc64_scene* S, const ray64* r, const hd64* hd, const hd64* he, d3 p, double* pdf,
                        float r1) {
  const orc_scene* s = S->s;
  if (s->nlights <= 0) { *pdf = 0; return D(0, 0, 0); }
  *pdf = s->nlights / (2.0 * PI64);
  int32_t li = f2i_dev((float)s->nlights * r1);
  if (li > s->nlights - 1) li = s->nlights - 1;
  const er_point_light* L = &s->lights[li];
  d3 lp = D(L->position[0], L->position[1], L->position[2]);
  d3 dir = nrm(sub(lp, p));
  double dist = len(sub(lp, p));
  ray64 sr = make_ray(add(p, scl(dir, 0.001)), dir);
  hit64 sh = closest(S, &sr);
  if (sh.valid && len(sub(sh.position, p)) < dist) return D(0, 0, 0);
  d3 plv = dvs(D(L->radiance[0], L->radiance[1], L->radiance[2]), dist * dist);
  d3 f = disney_eval64(r, he, dir);
  return dvs(scl(mul(plv, f), fabs(dot(dir, hd->normal))), *pdf);
}

/* kernel.cu:210-258, texel chosen as the FP32 renderers choose it */
static d3 hdri_light64(const orc64_scene* S, const ray64* r, d3 p, const hd64* hd, const hd64* he, const eval64* ev,
                       float r1, double* pdf) {
  const orc_scene* s = S->s;
  const orc_tex* t = &s->env;
  int32_t count = orc_hdri_search(s->cdf, r1, t->w * t->h);
  double nu = (double)(count % t->w) / t->w, nv = (double)(count / t->w) / t->h;
  int32_t x = d2i(nu * t->w), y = d2i(nv * t->h);
  x = d2i(t->xTile * ((double)x - (double)t->xOffset * t->w)) % t->w;
  y = d2i(t->yTile * ((double)y - (double)t->yOffset * t->h)) % t->h;
  double iu = (double)x / t->w, iv = (double)y / t->h;
  limit_uv64(&iu, &iv);
  d3 dir = scl(nrm(reverse_spherical64(iu, iv)), -1.0);
  int32_t px = d2i(iu * t->w), py = d2i(iv * t->h);
  d3 dv = Df(orc_tex_coord(t, px, py));
  double theta = ((double)py / t->h) * PI64;
  *pdf = ((dv.x + dv.y + dv.z) / S->radiance_sum) * t->w * t->h / (2.0 * PI64 * sin(theta));
  ray64 sr = make_ray(add(p, scl(dir, 0.001)), dir);
  hit64 sh = closest(S, &sr);
  if (sh.valid) return D(0, 0, 0);
  d3 hv = env_value64(t, ev, iu, iv);
  d3 f = disney_eval64(r, he, dir);
  return dvs(mul(scl(f, fabs(dot(dir, hd->normal))), hv), *pdf);
}

/* One sample (kernel.cu:369-443); returns the radiance before the clamp. */
static d3 sample64(const orc64_scene* S, int32_t x, int32_t y, uint32_t idx, uint32_t sample, int32_t max_depth,
                   uint32_t k0, uint32_t k1, const eval64* ev) {
  const orc_scene* s = S->s;
  uint32_t q[4];
  double cu[5];
  orc_philox(idx, sample, 0, 0, k0, k1, q);
  for (int k = 0; k < 4; k++) cu[k] = orc_u01(q[k]);
  orc_philox(idx, sample, 1, 0, k0, k1, q);
  cu[4] = orc_u01(q[0]);
  ray64 ray = camera64(&s->cam, x, y, cu);
  d3 light = D(0, 0, 0), red = D(1, 1, 1);
  for (int32_t i = 0; i < max_depth; i++) {
    hit64 hit = closest(S, &ray);
    if (!hit.valid) {
      double eu, ev_;
      spherical64(scl(ray.d, -1.0), &eu, &ev_);
      light = add(light, mul(env_value64(&s->env, ev, eu, ev_), red));
      break;
    }
    hd64 hd, he;
    const int32_t mid = s->tri_mat[hit.id];
    hit_data64(s, &s->mats[mid], &hit, &hd);
    hit_data_eval64(&s->mats[mid], mid, ev, &hd, &he);
    orc_philox(idx, sample, 2u + (uint32_t)i, 0, k0, k1, q);
    float r1 = orc_u01(q[3]);
    d3 dir = disney_sample64(&ray, &hd, orc_u01(q[0]), orc_u01(q[1]), orc_u01(q[2]));
    d3 f = disney_eval64(&ray, &he, dir);
    double brdfPdf = disney_pdf64(&ray, &hd, dir);
    double hdriPdf, pointPdf = 0;
    d3 hdriC = hdri_light64(S, &ray, hit.position, &hd, &he, ev, r1, &hdriPdf);
    d3 pointC = point_light64(S, &ray, &hd, &he, hit.position, &pointPdf, r1);
    d3 brdfC = dvs(mul(scl(f, fabs(dot(dir, hd.normal))), hd.emission), brdfPdf);
    double den = hdriPdf + pointPdf + brdfPdf;
    d3 hl = mul(add(add(scl(hdriC, hdriPdf / den), scl(pointC, pointPdf / den)), scl(brdfC, brdfPdf / den)), red);
    red = mul(red, dvs(scl(f, fabs(dot(dir, hd.normal))), brdfPdf));
    light = add(light, hl);
    ray = make_ray(add(hit.position, scl(dir, 0.001)), dir);
  }
  return light;
}

/* Mean over spp samples of the pixels with output indices idx[0..n):
 * rgb[3*i..] = mean of clamp(L, 0, 10) over non-NaN samples, counts[i] =
 * their number (kernel.cu:445-449). */
void orc64_render_pixels_eval(const orc64_scene* S, const int32_t* idx, int64_t n, int32_t spp, int32_t sample_begin,
                              int32_t max_depth, uint64_t seed, const float* eval_mat, const float* eval_env,
                              double* rgb, uint32_t* counts, int32_t nthreads) {
  const eval64 evs = {eval_mat, eval_env};
  const eval64* ev = (eval_mat || eval_env) ? &evs : NULL;
  const er_camera* c = &S->s->cam;
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
#endif
  for (int64_t i = 0; i < n; i++) {
    const int32_t o = idx[i];
    const int32_t x = o % c->x_res, y = c->y_res - 1 - o / c->x_res;
    double sx = 0, sy = 0, sz = 0;
    uint32_t cnt = 0;
    for (int32_t k = 0; k < spp; k++) {
      d3 L = sample64(S, x, y, (uint32_t)o, (uint32_t)(sample_begin + k), max_depth, k0, k1, ev);
      double lx = clampd(L.x, 0, 10), ly = clampd(L.y, 0, 10), lz = clampd(L.z, 0, 10);
      if (lx != lx || ly != ly || lz != lz) continue;
      sx += lx; sy += ly; sz += lz;
      cnt++;
    }
    rgb[3 * i] = cnt ? sx / cnt : 0;
    rgb[3 * i + 1] = cnt ? sy / cnt : 0;
    rgb[3 * i + 2] = cnt ? sz / cnt : 0;
    counts[i] = cnt;
  }
}

void orc64_render_pixels(const orc64_scene* S, const int32_t* idx, int64_t n, int32_t spp, int32_t sample_begin,
                         int32_t max_depth, uint64_t seed, double* rgb, uint32_t* counts, int32_t nthreads) {
  orc64_render_pixels_eval(S, idx, n, spp, sample_begin, max_depth, seed, NULL, NULL, rgb, counts, nthreads);
}

/* Closest hit by this BVH for rays (n x 6: origin, direction; normalised
 * here): triangle id (-1 = none) and shading distance. */
void orc64_trace(const orc64_scene* S, const float* rays, int64_t n, int32_t* tri, double* dist, int32_t nthreads) {
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
#endif
  for (int64_t i = 0; i < n; i++) {
    const float* q = rays + 6 * i;
    ray64 r = make_ray(D(q[0], q[1], q[2]), D(q[3], q[4], q[5]));
    hit64 h = closest(S, &r);
    tri[i] = h.valid ? h.id : -1;
    dist[i] = h.valid ? len(sub(h.position, r.o)) : INFINITY;
  }
}
