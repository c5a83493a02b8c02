/* mks_synth.h -- seeded synthetic lattice fields (host code, header only).
 *
 * One definition of the benchmark's synthetic inputs, compiled into two
 * libraries: the product library (mks_fields.c, mks_gen_* in the C ABI) and
 * the CPU oracle (oracle/orc_synth.c, orc_gen_*), so that a process that
 * must not load the product library (the CPU reference arm of the
 * benchmark) builds bit-identical inputs.
 *
 * Geometry follows MILC's single-node layout (generic/layout_hyper_prime.c:
 * 509-520): lexicographic i = x + nx*(y + ny*(z + nz*t)); even sites
 * ((x+y+z+t) even) are stored first at i/2, odd sites at (i+V)/2.
 *
 * Random numbers: Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
 * random numbers: as easy as 1, 2, 3", SC'11), keyed by the seed and
 * countered by (lexicographic site, slot, stream), so fields do not depend
 * on the layout, the thread count or the device.  Gaussian deviates use
 * MILC's normalisation exp(-x^2) (variance 1/2, libraries/gaussrand.c).
 *
 * Thin links U = exp(i a H), H traceless Hermitian built from a complex
 * Gaussian 3x3 matrix A as H = (A + A^dag)/2 - tr(A + A^dag)/6.  The
 * exponential is a scaling-and-squaring Taylor series in FP64, followed by
 * Gram-Schmidt reunitarisation of the first two rows and row3 =
 * conj(row1 x row2), which makes det U = 1 to rounding.
 *
 * parity arguments use MILC's codes: 0x02 even, 0x01 odd, 0x03 both.
 */
#ifndef MKS_SYNTH_H
#define MKS_SYNTH_H
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <stddef.h>

/* ---------------- Philox-4x32-10 ---------------- */
static inline void synth_mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

static void synth_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; r++) {
    uint32_t hi0, lo0, hi1, lo1;
    synth_mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
    synth_mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* A stream of gaussians for one (site, slot, stream); draw-indexed. */
typedef struct {
  uint32_t key[2];
  uint32_t ctr[4];
  uint32_t buf[4];
  int have;           /* number of unused 32-bit words left in buf */
} synth_rng;

static void synth_rng_init(synth_rng *r, uint64_t seed, uint64_t site, uint32_t slot, uint32_t stream) {
  r->key[0] = (uint32_t)seed;
  r->key[1] = (uint32_t)(seed >> 32);
  r->ctr[0] = 0;                       /* draw counter */
  r->ctr[1] = (uint32_t)site;
  r->ctr[2] = (uint32_t)(site >> 32) ^ (slot << 16);
  r->ctr[3] = stream;
  r->have = 0;
}

static uint32_t synth_u32(synth_rng *r) {
  if (r->have == 0) {
    synth_philox4x32_10(r->ctr, r->key, r->buf);
    r->ctr[0]++;
    r->have = 4;
  }
  return r->buf[4 - (r->have--)];
}

/* uniform in (0,1]: 53 random bits */
static double synth_uniform(synth_rng *r) {
  uint32_t a = synth_u32(r) >> 5, b = synth_u32(r) >> 6;
  double u = ((double)a * 67108864.0 + (double)b) * (1.0 / 9007199254740992.0);
  return 1.0 - u;
}

/* gaussian with <x^2> = 1/2 (weight exp(-x^2)), Box-Muller */
static double synth_gauss(synth_rng *r) {
  double u1 = synth_uniform(r), u2 = synth_uniform(r);
  return sqrt(-log(u1)) * cos(6.283185307179586476925286766559 * u2);
}

/* ---------------- geometry ---------------- */
static void synth_site_coords(const int dims[4], size_t index, int xyzt[4]) {
  size_t V = (size_t)dims[0] * dims[1] * dims[2] * dims[3];
  size_t half = V / 2;
  int parity = index >= half;          /* 0 even, 1 odd */
  size_t h = parity ? index - half : index;
  /* lexicographic i has i/2 == h; the two candidates 2h and 2h+1 differ by
     one step in x (nx even), exactly one has the requested parity */
  size_t i = 2 * h;
  int x = (int)(i % dims[0]);
  size_t r = i / dims[0];
  int y = (int)(r % dims[1]); r /= dims[1];
  int z = (int)(r % dims[2]);
  int t = (int)(r / dims[2]);
  if (((x + y + z + t) & 1) != parity) x += 1;
  xyzt[0] = x; xyzt[1] = y; xyzt[2] = z; xyzt[3] = t;
}

static inline size_t synth_lex(const int dims[4], const int c[4]) {
  return (size_t)c[0] + (size_t)dims[0] * ((size_t)c[1] + (size_t)dims[1] *
         ((size_t)c[2] + (size_t)dims[2] * (size_t)c[3]));
}

/* ---------------- 3x3 complex helpers (row-major, interleaved re/im) ---------------- */
typedef struct { double e[3][3][2]; } synth_m3;

static void synth_m3_mul(const synth_m3 *a, const synth_m3 *b, synth_m3 *c) {
  synth_m3 r;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double re = 0, im = 0;
      for (int k = 0; k < 3; k++) {
        re += a->e[i][k][0] * b->e[k][j][0] - a->e[i][k][1] * b->e[k][j][1];
        im += a->e[i][k][0] * b->e[k][j][1] + a->e[i][k][1] * b->e[k][j][0];
      }
      r.e[i][j][0] = re; r.e[i][j][1] = im;
    }
  *c = r;
}

static double synth_m3_norm1(const synth_m3 *a) {
  double s = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) s += hypot(a->e[i][j][0], a->e[i][j][1]);
  return s;
}

/* exp(M) by scaling and squaring with a degree-18 Taylor polynomial */
static void synth_m3_exp(const synth_m3 *M, synth_m3 *E) {
  double nrm = synth_m3_norm1(M);
  int s = 0;
  while (nrm > 0.25 && s < 60) { nrm *= 0.5; s++; }
  double scale = ldexp(1.0, -s);
  synth_m3 A;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      A.e[i][j][0] = M->e[i][j][0] * scale;
      A.e[i][j][1] = M->e[i][j][1] * scale;
    }
  /* Horner: E = I + A(I + A/2(I + A/3(...))) */
  synth_m3 R;
  memset(&R, 0, sizeof R);
  for (int i = 0; i < 3; i++) R.e[i][i][0] = 1.0;
  for (int k = 18; k >= 1; k--) {
    synth_m3 T;
    synth_m3_mul(&A, &R, &T);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        R.e[i][j][0] = T.e[i][j][0] / k + (i == j ? 1.0 : 0.0);
        R.e[i][j][1] = T.e[i][j][1] / k;
      }
  }
  for (int q = 0; q < s; q++) synth_m3_mul(&R, &R, &R);
  *E = R;
}

/* Gram-Schmidt on rows 0,1; row 2 = conj(row0 x row1): exactly SU(3) up to rounding */
static void synth_m3_reunit_su3(synth_m3 *U) {
  double n0 = 0;
  for (int j = 0; j < 3; j++) n0 += U->e[0][j][0] * U->e[0][j][0] + U->e[0][j][1] * U->e[0][j][1];
  n0 = 1.0 / sqrt(n0);
  for (int j = 0; j < 3; j++) { U->e[0][j][0] *= n0; U->e[0][j][1] *= n0; }
  /* c = <row0|row1> */
  double cr = 0, ci = 0;
  for (int j = 0; j < 3; j++) {
    cr += U->e[0][j][0] * U->e[1][j][0] + U->e[0][j][1] * U->e[1][j][1];
    ci += U->e[0][j][0] * U->e[1][j][1] - U->e[0][j][1] * U->e[1][j][0];
  }
  for (int j = 0; j < 3; j++) {
    U->e[1][j][0] -= cr * U->e[0][j][0] - ci * U->e[0][j][1];
    U->e[1][j][1] -= cr * U->e[0][j][1] + ci * U->e[0][j][0];
  }
  double n1 = 0;
  for (int j = 0; j < 3; j++) n1 += U->e[1][j][0] * U->e[1][j][0] + U->e[1][j][1] * U->e[1][j][1];
  n1 = 1.0 / sqrt(n1);
  for (int j = 0; j < 3; j++) { U->e[1][j][0] *= n1; U->e[1][j][1] *= n1; }
  /* row2 = conj(row0 x row1) */
  for (int j = 0; j < 3; j++) {
    int a = (j + 1) % 3, b = (j + 2) % 3;
    double re = U->e[0][a][0] * U->e[1][b][0] - U->e[0][a][1] * U->e[1][b][1]
              - (U->e[0][b][0] * U->e[1][a][0] - U->e[0][b][1] * U->e[1][a][1]);
    double im = U->e[0][a][0] * U->e[1][b][1] + U->e[0][a][1] * U->e[1][b][0]
              - (U->e[0][b][0] * U->e[1][a][1] + U->e[0][b][1] * U->e[1][a][0]);
    U->e[2][j][0] = re;
    U->e[2][j][1] = -im;
  }
}

/* Stream identifiers keep the different synthetic fields independent. */
enum { SYNTH_STREAM_LINKS = 1, SYNTH_STREAM_VECTOR = 2, SYNTH_STREAM_MOM = 3 };

static int synth_dims_ok(const int dims[4]) {
  if (!dims) return 0;
  for (int d = 0; d < 4; d++)
    if (dims[d] <= 0 || (dims[d] & 1)) return 0;
  return 1;
}

/* thin links U[V][4][18] = exp(i a H) per (site, dir), no phases */
static void synth_thin_links(const int dims[4], uint64_t seed, double a, double *links) {
  size_t V = (size_t)dims[0] * dims[1] * dims[2] * dims[3];
  long long n = (long long)V;
#pragma omp parallel for schedule(static)
  for (long long idx = 0; idx < n; idx++) {
    int c[4];
    synth_site_coords(dims, (size_t)idx, c);
    size_t lex = synth_lex(dims, c);
    for (int dir = 0; dir < 4; dir++) {
      synth_rng r;
      synth_rng_init(&r, seed, lex, (uint32_t)dir, SYNTH_STREAM_LINKS);
      synth_m3 A, H, M, U;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) { A.e[i][j][0] = synth_gauss(&r); A.e[i][j][1] = synth_gauss(&r); }
      double tr = 0;
      for (int i = 0; i < 3; i++) tr += A.e[i][i][0];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          H.e[i][j][0] = 0.5 * (A.e[i][j][0] + A.e[j][i][0]);
          H.e[i][j][1] = 0.5 * (A.e[i][j][1] - A.e[j][i][1]);
        }
      for (int i = 0; i < 3; i++) H.e[i][i][0] -= tr / 3.0;
      /* M = i a H */
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          M.e[i][j][0] = -a * H.e[i][j][1];
          M.e[i][j][1] = a * H.e[i][j][0];
        }
      synth_m3_exp(&M, &U);
      synth_m3_reunit_su3(&U);
      memcpy(links + ((size_t)idx * 4 + dir) * 18, &U, 18 * sizeof(double));
    }
  }
}

/* Gaussian colour vector [V][6] on the sites of `parity`, zero elsewhere */
static void synth_vector(const int dims[4], uint64_t seed, int parity, double *vec) {
  size_t V = (size_t)dims[0] * dims[1] * dims[2] * dims[3];
  long long n = (long long)V;
#pragma omp parallel for schedule(static)
  for (long long idx = 0; idx < n; idx++) {
    int c[4];
    synth_site_coords(dims, (size_t)idx, c);
    int p = (c[0] + c[1] + c[2] + c[3]) & 1;      /* 0 = even */
    double *v = vec + (size_t)idx * 6;
    int want = (parity == 0x03) || (parity == 0x02 && p == 0) || (parity == 0x01 && p == 1);
    if (!want) { for (int k = 0; k < 6; k++) v[k] = 0.0; continue; }
    synth_rng r;
    synth_rng_init(&r, seed, synth_lex(dims, c), 0, SYNTH_STREAM_VECTOR);
    for (int k = 0; k < 6; k++) v[k] = synth_gauss(&r);
  }
}

/* Gaussian anti-Hermitian traceless momenta [V][4][10] in MILC's
   anti_hermitmat order (m01, m02, m12 complex, m00im, m11im, m22im, space) */
static void synth_momenta(const int dims[4], uint64_t seed, double *mom) {
  size_t V = (size_t)dims[0] * dims[1] * dims[2] * dims[3];
  long long n = (long long)V;
#pragma omp parallel for schedule(static)
  for (long long idx = 0; idx < n; idx++) {
    int c[4];
    synth_site_coords(dims, (size_t)idx, c);
    for (int dir = 0; dir < 4; dir++) {
      synth_rng r;
      synth_rng_init(&r, seed, synth_lex(dims, c), (uint32_t)dir, SYNTH_STREAM_MOM);
      double *m = mom + ((size_t)idx * 4 + dir) * 10;
      double g[8];
      for (int k = 0; k < 8; k++) g[k] = synth_gauss(&r);
      m[0] = g[0]; m[1] = g[1]; m[2] = g[2]; m[3] = g[3]; m[4] = g[4]; m[5] = g[5];
      /* traceless diagonal: a, b, -(a+b) scaled like MILC's random_anti_hermitian */
      double d1 = g[6], d2 = g[7] * 0.57735026918962576451;
      m[6] = d1 + d2; m[7] = -d1 + d2; m[8] = -2.0 * d2; m[9] = 0.0;
    }
  }
}

#endif /* MKS_SYNTH_H */
