/* rscape_oracle.c -- CPU FP64 restatement of R-scape's covariation path.
 *
 * TEST INFRASTRUCTURE ONLY (see rscape_oracle.h).  Each function names the
 * reference file:line it follows.  Easel routines that the reference calls
 * but that are absent from the reference tree (histograms, binned fits,
 * weights, RNG) are restated from their published mathematics and marked
 * "restated".
 */
#include "rscape_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define K4   4
#define K16 16
#define ORC_GAP 4
#define ORC_N   15
#define IS_CANON(x) ((x) < 4)

/* ------------------------------------------------------------------ */
/* RNG: Philox4x32-10, Salmon, Moraes, Dror, Shaw, "Parallel random    */
/* numbers: as easy as 1, 2, 3", SC'11.                                */
/* ------------------------------------------------------------------ */
void
orc_philox4x32(const uint32_t key[2], const uint32_t ctr[4], uint32_t out[4])
{
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  int r;
  for (r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* stream tags of the null-alignment generator and of the simulator */
#define TAG_FLEAF   0x11u
#define TAG_FCHOOSE 0x12u
#define TAG_COLPERM 0x13u
#define TAG_SUBST   0x14u
#define TAG_SIMROOT 0x21u
#define TAG_SIMSUB  0x22u
#define TAG_SIMGAP  0x23u

static uint32_t
rng_u32(uint64_t seed, uint32_t tag, uint32_t null_id, uint32_t a, uint32_t b)
{
  uint32_t key[2] = { (uint32_t)seed, (uint32_t)(seed >> 32) };
  uint32_t ctr[4] = { tag, null_id, a, b };
  uint32_t out[4];
  orc_philox4x32(key, ctr, out);
  return out[0];
}

static uint64_t
rng_u64(uint64_t seed, uint32_t tag, uint32_t rep, uint32_t a, uint32_t b)
{
  uint32_t key[2] = { (uint32_t)seed, (uint32_t)(seed >> 32) };
  uint32_t ctr[4] = { tag, rep, a, b };
  uint32_t out[4];
  orc_philox4x32(key, ctr, out);
  return (uint64_t)out[0] | ((uint64_t)out[1] << 32);
}

static void
rng_round_keys(uint64_t seed, uint32_t tag, uint32_t null_id, uint32_t idx, uint32_t rk[6])
{
  uint32_t key[2] = { (uint32_t)seed, (uint32_t)(seed >> 32) };
  uint32_t ctr[4] = { tag, null_id, idx, 0 };
  uint32_t out[4];
  orc_philox4x32(key, ctr, out);
  rk[0] = out[0]; rk[1] = out[1]; rk[2] = out[2]; rk[3] = out[3];
  ctr[3] = 1;
  orc_philox4x32(key, ctr, out);
  rk[4] = out[0]; rk[5] = out[1];
}

static uint32_t
fmix32(uint32_t h)
{ /* MurmurHash3 finalizer (Appleby, public domain) */
  h ^= h >> 16; h *= 0x85EBCA6Bu;
  h ^= h >> 13; h *= 0xC2B2AE35u;
  h ^= h >> 16;
  return h;
}

/* Random permutation of [0,L) as a 6-round balanced Feistel network on the
 * smallest even-bit domain >= L, with cycle walking (Black & Rogaway 2002). */
uint32_t
orc_feistel_perm(uint32_t t, uint32_t L, const uint32_t rk[6])
{
  uint32_t h = 1, mask, x = t;
  int r;
  while ((1u << (2 * h)) < L) h++;
  mask = (1u << h) - 1u;
  do {
    uint32_t l = x >> h, rr = x & mask;
    for (r = 0; r < 6; r++) {
      uint32_t nl = rr;
      uint32_t nr = l ^ (fmix32(rr ^ rk[r]) & mask);
      l = nl; rr = nr;
    }
    x = (l << h) | rr;
  } while (x >= L);
  return x;
}

/* ------------------------------------------------------------------ */
/* vector helpers (Easel esl_vec_DNorm / DValidate restated)           */
/* ------------------------------------------------------------------ */
static void
vec_norm(double *v, int n)
{
  double sum = 0.0;
  int i;
  for (i = 0; i < n; i++) sum += v[i];
  if (sum != 0.0) for (i = 0; i < n; i++) v[i] /= sum;
  else            for (i = 0; i < n; i++) v[i] = 1.0 / (double)n;
}

static int
vec_validate(const double *v, int n, double tol)
{
  double sum = 0.0;
  int i;
  for (i = 0; i < n; i++) {
    if (!(v[i] >= 0.0 && v[i] <= 1.0 + tol)) return 1;
    sum += v[i];
  }
  return (fabs(sum - 1.0) > tol) ? 1 : 0;
}

/* ------------------------------------------------------------------ */
/* MSA preparation                                                     */
/* ------------------------------------------------------------------ */

/* msamanip_ConvertDegen2N + ConvertMissingNonresidue2Gap
 * (called at src/R-scape.c:1855-1856): degenerate codes -> N, '*','~' -> gap */
void
orc_degen2n(uint8_t *ax, int64_t n)
{
  int64_t i;
  for (i = 0; i < n; i++) {
    if (ax[i] > ORC_GAP && ax[i] < ORC_N) ax[i] = ORC_N;
    else if (ax[i] > ORC_N)               ax[i] = ORC_GAP;
  }
}

/* msamanip_RemoveGapColumns, src/msamanip.c:461-501: keep a column iff its
 * weighted residue fraction (residues over residues+gaps) >= 1-gapthresh. */
int
orc_gapfilter(const uint8_t *ax, const double *wgt, int N, int L, double gapthresh, int *useme)
{
  double idthresh = 1.0 - gapthresh;
  int s, c;
  for (c = 0; c < L; c++) {
    double r = 0.0, tot = 0.0;
    for (s = 0; s < N; s++) {
      uint8_t x = ax[(int64_t)s * L + c];
      double  w = wgt ? wgt[s] : 1.0;
      if (x < ORC_GAP || (x > ORC_GAP && x <= ORC_N)) { r += w; tot += w; }
      else if (x == ORC_GAP || x == 16)               { tot += w; }
      /* '~' (missing) is skipped */
    }
    useme[c] = (r > 0.0 && r / tot >= idthresh) ? 1 : 0;
  }
  return 0;
}

/* Position-based weights (Henikoff & Henikoff, J Mol Biol 243:574, 1994),
 * restated; called at src/R-scape.c:1556 for nseq > 1000.  Canonical residues
 * only; weights renormalised to sum to N. */
int
orc_weights_pb(const uint8_t *ax, int N, int L, double *wgt)
{
  int s, c, x;
  double sum = 0.0;
  for (s = 0; s < N; s++) wgt[s] = 0.0;
  for (c = 0; c < L; c++) {
    int cnt[4] = { 0, 0, 0, 0 }, ntypes = 0;
    for (s = 0; s < N; s++) { x = ax[(int64_t)s * L + c]; if (IS_CANON(x)) cnt[x]++; }
    for (x = 0; x < 4; x++) if (cnt[x] > 0) ntypes++;
    if (ntypes == 0) continue;
    for (s = 0; s < N; s++) {
      x = ax[(int64_t)s * L + c];
      if (IS_CANON(x)) wgt[s] += 1.0 / ((double)ntypes * (double)cnt[x]);
    }
  }
  for (s = 0; s < N; s++) sum += wgt[s];
  if (sum > 0.0) for (s = 0; s < N; s++) wgt[s] *= (double)N / sum;
  else           for (s = 0; s < N; s++) wgt[s] = 1.0;
  return 0;
}

/* Gerstein/Sonnhammer/Chothia tree weights (J Mol Biol 236:1067, 1994),
 * restated; called at src/R-scape.c:1555 for nseq <= 1000.
 * Distances: 1 - identities/min(residues_a, residues_b) over columns where
 * both sequences carry a residue.  Tree: UPGMA.  Weights: going up the tree,
 * each leaf starts with its own branch length; the branch above each
 * internal node is shared among the leaves below it in proportion to their
 * current weights (equally when those are all zero).  Normalised to sum N. */
int
orc_weights_gsc(const uint8_t *ax, int N, int L, double *wgt)
{
  double *D = NULL, *height = NULL, sum;
  int    *size = NULL, *alive = NULL, *node = NULL, *len = NULL;
  int   **members = NULL;
  int    *nmem = NULL;
  int     a, b, c, s, k, nclust;

  if (N == 1) { wgt[0] = 1.0; return 0; }
  D       = malloc(sizeof(double) * N * N);
  height  = calloc(N, sizeof(double));
  size    = malloc(sizeof(int) * N);
  alive   = malloc(sizeof(int) * N);
  len     = calloc(N, sizeof(int));
  members = malloc(sizeof(int *) * N);
  nmem    = malloc(sizeof(int) * N);
  node    = NULL;
  if (!D || !height || !size || !alive || !len || !members || !nmem) return 1;

  for (s = 0; s < N; s++)
    for (c = 0; c < L; c++) { uint8_t x = ax[(int64_t)s * L + c]; if (x < ORC_GAP || (x > ORC_GAP && x <= ORC_N)) len[s]++; }
  for (a = 0; a < N; a++) {
    D[a * N + a] = 0.0;
    for (b = a + 1; b < N; b++) {
      int idents = 0, mn = (len[a] < len[b]) ? len[a] : len[b];
      for (c = 0; c < L; c++) {
        uint8_t x = ax[(int64_t)a * L + c], y = ax[(int64_t)b * L + c];
        int rx = (x < ORC_GAP || (x > ORC_GAP && x <= ORC_N));
        int ry = (y < ORC_GAP || (y > ORC_GAP && y <= ORC_N));
        if (rx && ry && x == y) idents++;
      }
      D[a * N + b] = D[b * N + a] = (mn == 0) ? 1.0 : 1.0 - (double)idents / (double)mn;
    }
  }
  for (s = 0; s < N; s++) {
    size[s] = 1; alive[s] = 1; wgt[s] = 0.0;
    members[s] = malloc(sizeof(int) * N); members[s][0] = s; nmem[s] = 1;
  }
  /* UPGMA; every leaf's branch is counted when its cluster first merges */
  nclust = N;
  while (nclust > 1) {
    double best = DBL_MAX, h, bl_a, bl_b, tot_a = 0.0, tot_b = 0.0;
    int ba = -1, bb = -1;
    for (a = 0; a < N; a++) if (alive[a])
      for (b = a + 1; b < N; b++) if (alive[b])
        if (D[a * N + b] < best) { best = D[a * N + b]; ba = a; bb = b; }
    h    = best / 2.0;
    bl_a = h - height[ba]; if (bl_a < 0.0) bl_a = 0.0;
    bl_b = h - height[bb]; if (bl_b < 0.0) bl_b = 0.0;
    /* branch above cluster ba (length bl_a) is shared by its leaves */
    for (k = 0; k < nmem[ba]; k++) tot_a += wgt[members[ba][k]];
    for (k = 0; k < nmem[bb]; k++) tot_b += wgt[members[bb][k]];
    for (k = 0; k < nmem[ba]; k++) {
      int l = members[ba][k];
      wgt[l] += (tot_a > 0.0) ? bl_a * wgt[l] / tot_a : bl_a / (double)nmem[ba];
    }
    for (k = 0; k < nmem[bb]; k++) {
      int l = members[bb][k];
      wgt[l] += (tot_b > 0.0) ? bl_b * wgt[l] / tot_b : bl_b / (double)nmem[bb];
    }
    /* merge bb into ba */
    for (c = 0; c < N; c++) if (alive[c] && c != ba && c != bb) {
      double d = (D[ba * N + c] * size[ba] + D[bb * N + c] * size[bb]) / (double)(size[ba] + size[bb]);
      D[ba * N + c] = D[c * N + ba] = d;
    }
    for (k = 0; k < nmem[bb]; k++) members[ba][nmem[ba]++] = members[bb][k];
    size[ba] += size[bb];
    height[ba] = h;
    alive[bb] = 0;
    nclust--;
  }
  sum = 0.0;
  for (s = 0; s < N; s++) sum += wgt[s];
  if (sum > 0.0) for (s = 0; s < N; s++) wgt[s] *= (double)N / sum;
  else           for (s = 0; s < N; s++) wgt[s] = 1.0;

  for (s = 0; s < N; s++) free(members[s]);
  free(members); free(nmem); free(D); free(height); free(size); free(alive); free(len); free(node);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Probabilities                                                       */
/* ------------------------------------------------------------------ */

/* mutual_naive_ppij, src/correlators.c:1695-1780 (GAPASCHAR 0 branch,
 * :1745-1752): prior 1e-10 per cell, nseff over both-canonical rows, ngap
 * over the rest; normalise; mirror pp and nseff (ngap is not mirrored). */
static void
naive_ppij(const uint8_t *ax, const double *wgt, int N, int L, int i, int j,
           double *pp, double *nseff, double *ngap)
{
  double *p = pp + ((int64_t)i * L + j) * K16;
  double  ne = 0.0, ng = 0.0;
  int     s, x, y;
  for (x = 0; x < K16; x++) p[x] = 1e-10;
  for (s = 0; s < N; s++) {
    int ri = ax[(int64_t)s * L + i], rj = ax[(int64_t)s * L + j];
    if (IS_CANON(ri) && IS_CANON(rj)) { ne += wgt[s]; p[ri * K4 + rj] += wgt[s]; }
    else                              { ng += wgt[s]; }
  }
  vec_norm(p, K16);
  for (x = 0; x < K4; x++)
    for (y = 0; y < K4; y++)
      pp[((int64_t)j * L + i) * K16 + y * K4 + x] = p[x * K4 + y];
  nseff[(int64_t)i * L + j] = nseff[(int64_t)j * L + i] = ne;
  ngap[(int64_t)i * L + j] = ng;
}

/* corr_Probs NONPARAM (src/correlators.c:1423-1496): NaivePP (:1300),
 * NaivePS (:1319, psi at :1782-1817, prior 1e-5 over K+1 = 5 bins),
 * Marginals (:1337-1375), ValidateProbs (:1499-1545). */
int
orc_probs(const uint8_t *ax, const double *wgt, int N, int L, double tol,
          double *pp, double *nseff, double *ngap, double *pm, double *ps)
{
  int i, j, x, y, s;

  memset(pp,    0, sizeof(double) * (size_t)L * L * K16);
  memset(nseff, 0, sizeof(double) * (size_t)L * L);
  memset(ngap,  0, sizeof(double) * (size_t)L * L);

  if ((double)N * L * L < 4e9) {
    for (i = 0; i < L - 1; i++)
      for (j = i + 1; j < L; j++)
        naive_ppij(ax, wgt, N, L, i, j, pp, nseff, ngap);
  } else {
    /* deep alignments: the same sums (sequence order per pair) from a
     * column-major copy, pairs spread over the host threads */
    /* column-major codes folded to 0..3 (canonical) and 4 (anything
     * else); each pair's weights then go to a 5x5 table without branches,
     * every cell summing its sequences' weights in sequence order */
    uint8_t *axT = malloc((size_t)N * L);
    if (!axT) return 5;
    for (s = 0; s < N; s++)
      for (i = 0; i < L; i++) {
        const int r = ax[(size_t)s * L + i];
        axT[(size_t)i * N + s] = (uint8_t)(IS_CANON(r) ? r : K4);
      }
#pragma omp parallel for schedule(dynamic, 1) private(j, x, y, s)
    for (i = 0; i < L - 1; i++) {
      const uint8_t *ci = axT + (size_t)i * N;
      for (j = i + 1; j < L; j++) {
        const uint8_t *cj = axT + (size_t)j * N;
        double *p = pp + ((int64_t)i * L + j) * K16;
        double  ne = 0.0, ng = 0.0, c[25];
        for (x = 0; x < 25; x++) c[x] = 0.0;
        for (s = 0; s < N; s++) c[ci[s] * 5 + cj[s]] += wgt[s];
        for (x = 0; x < 25; x++) {
          if (x % 5 < K4 && x / 5 < K4) ne += c[x];
          else                          ng += c[x];
        }
        for (x = 0; x < K4; x++)
          for (y = 0; y < K4; y++) p[x * K4 + y] = 1e-10 + c[x * 5 + y];
        vec_norm(p, K16);
        for (x = 0; x < K4; x++)
          for (y = 0; y < K4; y++)
            pp[((int64_t)j * L + i) * K16 + y * K4 + x] = p[x * K4 + y];
        nseff[(int64_t)i * L + j] = nseff[(int64_t)j * L + i] = ne;
        ngap[(int64_t)i * L + j] = ng;
      }
    }
    free(axT);
  }

  for (i = 0; i < L; i++) {
    double *q = ps + (int64_t)i * 5;
    for (x = 0; x < 5; x++) q[x] = 1e-5;
    for (s = 0; s < N; s++) { int r = ax[(int64_t)s * L + i]; if (r < 5) q[r] += wgt[s]; }
    vec_norm(q, 5);
  }

  for (i = 0; i < L; i++) {
    double *m = pm + (int64_t)i * K4;
    for (x = 0; x < K4; x++) m[x] = 0.0;
    for (x = 0; x < K4; x++)
      for (j = 0; j < L; j++)
        for (y = 0; y < K4; y++)
          if (nseff[(int64_t)i * L + j] > 0) m[x] += pp[((int64_t)i * L + j) * K16 + x * K4 + y];
    vec_norm(m, K4);
    if (vec_validate(m, K4, tol)) return 2;
  }

  for (i = 0; i < L - 1; i++)
    for (j = i + 1; j < L; j++)
      if (vec_validate(pp + ((int64_t)i * L + j) * K16, K16, tol)) return 3;
  for (i = 0; i < L; i++)
    if (vec_validate(ps + (int64_t)i * 5, 5, tol)) return 4;
  return 0;
}

/* ------------------------------------------------------------------ */
/* Statistics                                                          */
/* ------------------------------------------------------------------ */

static int
is_allowed(int x, int y, const double *allow)
{ /* is_allowed_pair, src/correlators.c:1669-1674 */
  return (x < 4 && y < 4 && allow[x * 4 + y] > 0) ? 1 : 0;
}

static void
cov_reset(int L, double *COV, double *minmax)
{ /* corr_ReuseCOV, src/correlators.c:1254-1268 */
  int64_t k;
  for (k = 0; k < (int64_t)L * L; k++) COV[k] = -INFINITY;
  minmax[0] = INFINITY; minmax[1] = -INFINITY;
}

static void
cov_set(int L, double *COV, double *minmax, int i, int j, double v)
{
  COV[(int64_t)i * L + j] = COV[(int64_t)j * L + i] = v;
  if (v < minmax[0]) minmax[0] = v;
  if (v > minmax[1]) minmax[1] = v;
}

/* one pair, C16 class: CHI :92-122, OMES :224-252, GT :359-390, MI :536-561,
 * MIr :659-690, MIg :792-822 */
static double
pair_c16(int stat, double ne, double ng, const double *p, const double *mi, const double *mj)
{
  double v = 0.0, HH = 0.0;
  int x, y;
  for (x = 0; x < K4; x++)
    for (y = 0; y < K4; y++) {
      double pxy = p[x * K4 + y];
      double exp = ne * mi[x] * mj[y];
      double obs = ne * pxy;
      switch (stat) {
      case ORC_CHI:  v += (exp > 0.) ? (obs - exp) * (obs - exp) / exp : 0.0; break;
      case ORC_OMES: v += (exp > 0.) ? (obs - exp) * (obs - exp) / ne : 0.0; break;
      case ORC_GT:   v += (exp > 0. && obs > 0.) ? obs * log(obs / exp) : 0.0; break;
      case ORC_MI: case ORC_MIg:
        v += (pxy > 0.0 && mi[x] > 0.0 && mj[y] > 0.0) ? pxy * (log(pxy) - log(mi[x]) - log(mj[y])) : 0.0; break;
      case ORC_MIr:
        HH -= (pxy > 0.0) ? pxy * log(pxy) : 0.0;
        v += (pxy > 0.0 && mi[x] > 0.0 && mj[y] > 0.0) ? pxy * (log(pxy) - log(mi[x]) - log(mj[y])) : 0.0; break;
      }
    }
  if (stat == ORC_GT)  v *= 2.0;
  if (stat == ORC_MIr) v = (HH > 1e-2) ? v / HH : 0.0;
  if (stat == ORC_MIg) v -= (ne > 0) ? ng / ne : 0.0;
  return v;
}

/* one pair, C2 class: CHI :137-168, OMES :269-301, GT :426-463, MI :575-605,
 * MIr :705-736, MIg :838-866 */
static double
pair_c2(int stat, double ne, double ng, const double *p, const double *mi, const double *mj, const double *allow)
{
  double pw = 0., pn = 0., qw = 0., qn = 0., v = 0.0, HH = 0.0;
  double ew, en, ow, on;
  int x, y;
  for (x = 0; x < K4; x++)
    for (y = 0; y < K4; y++) {
      if (is_allowed(x, y, allow)) { pw += p[x * K4 + y]; qw += mi[x] * mj[y]; }
      else                         { pn += p[x * K4 + y]; qn += mi[x] * mj[y]; }
    }
  ew = ne * qw; en = ne * qn; ow = ne * pw; on = ne * pn;
  switch (stat) {
  case ORC_CHI:
    v += (ew > 0.) ? (ow - ew) * (ow - ew) / ew : 0.0;
    v += (en > 0.) ? (on - en) * (on - en) / en : 0.0; break;
  case ORC_OMES:
    v += (ew > 0.) ? (ow - ew) * (ow - ew) / ne : 0.0;
    v += (en > 0.) ? (on - en) * (on - en) / ne : 0.0; break;
  case ORC_GT:
    v += (ew > 0. && ow > 0.) ? ow * log(ow / ew) : 0.0;
    v += (en > 0. && on > 0.) ? on * log(on / en) : 0.0;
    v *= 2.0; break;
  case ORC_MI: case ORC_MIg:
    v += (pw > 0.) ? pw * (log(pw) - log(qw)) : 0.0;
    v += (pn > 0.) ? pn * (log(pn) - log(qn)) : 0.0;
    if (stat == ORC_MIg) v -= (ne > 0) ? ng / ne : 0.0;
    break;
  case ORC_MIr:
    HH -= (pw > 0.) ? pw * log(pw) : 0.0;
    HH -= (pn > 0.) ? pn * log(pn) : 0.0;
    v += (pw > 0. && qw > 0.0) ? pw * (log(pw) - log(qw)) : 0.0;
    v += (pn > 0. && qn > 0.0) ? pn * (log(pn) - log(qn)) : 0.0;
    v = (HH > 1e-2) ? v / HH : 0.0; break;
  }
  return v;
}

/* GT CWC, src/correlators.c:393-423: allowed cells only */
static double
pair_gt_cwc(double ne, const double *p, const double *mi, const double *mj, const double *allow)
{
  double v = 0.0;
  int x, y;
  for (x = 0; x < K4; x++)
    for (y = 0; y < K4; y++)
      if (is_allowed(x, y, allow)) {
        double exp = ne * mi[x] * mj[y], obs = ne * p[x * K4 + y];
        v += (exp > 0. && obs > 0.) ? obs * log(obs / exp) : 0.0;
      }
  return 2.0 * v;
}

/* corr_Calculate{CHI,OMES,GT,MI,MIr,MIg} dispatchers with CSELECT
 * (e.g. src/correlators.c:58-68, 335-342): C2 when nseq <= nseqthresh or
 * alen <= alenthresh. */
int
orc_stat(int stat, int covclass, int N, int L, int nseqthresh, int alenthresh,
         const double *pp, const double *pm, const double *nseff, const double *ngap,
         const double *allow, double *COV, double *minmax)
{
  int i, j, cls = covclass;
  if (cls == ORC_CSELECT) cls = (N <= nseqthresh || L <= alenthresh) ? ORC_C2 : ORC_C16;
  if (cls == ORC_CWC && stat != ORC_GT) return 1;
  cov_reset(L, COV, minmax);
  /* pairs are independent: rows over the host threads, then min/max in order */
#pragma omp parallel for schedule(dynamic, 4) private(j)
  for (i = 0; i < L - 1; i++)
    for (j = i + 1; j < L; j++) {
      const double *p  = pp + ((int64_t)i * L + j) * K16;
      double        ne = nseff[(int64_t)i * L + j], ng = ngap[(int64_t)i * L + j], v;
      if      (cls == ORC_C16) v = pair_c16(stat, ne, ng, p, pm + i * K4, pm + j * K4);
      else if (cls == ORC_C2)  v = pair_c2 (stat, ne, ng, p, pm + i * K4, pm + j * K4, allow);
      else                     v = pair_gt_cwc(ne, p, pm + i * K4, pm + j * K4, allow);
      COV[(int64_t)i * L + j] = COV[(int64_t)j * L + i] = v;
    }
  for (i = 0; i < L - 1; i++)
    for (j = i + 1; j < L; j++) {
      const double v = COV[(int64_t)i * L + j];
      if (v < minmax[0]) minmax[0] = v;
      if (v > minmax[1]) minmax[1] = v;
    }
  return 0;
}

/* corr_CalculateRAF for deep alignments: the same sums from the unweighted
 * counts of the allowed cells.  Over the unordered pairs of sequences whose
 * residues at (i, j) are both allowed, the loop below adds [a_i != b_i] +
 * [a_j != b_j]; with n_A allowed sequences, r_x of them with x at i and c_y
 * with y at j, that is (n_A^2 - sum r_x^2)/2 + (n_A^2 - sum c_y^2)/2, an
 * integer formed exactly.  The pairs are spread over the host threads. */
int
orc_raf_counts(const uint8_t *ax, int N, int L, const double *allow, double *COV, double *minmax)
{
  uint8_t *axT = malloc((size_t)N * L);
  int      i, s;
  if (!axT) return 5;
  for (s = 0; s < N; s++)   /* codes folded to 0..3 and 4 (not canonical) */
    for (i = 0; i < L; i++) {
      const int r = ax[(size_t)s * L + i];
      axT[(size_t)i * N + s] = (uint8_t)(r < K4 ? r : K4);
    }
  cov_reset(L, COV, minmax);
#pragma omp parallel for schedule(dynamic, 1)
  for (i = 0; i < L - 1; i++) {
    const uint8_t *ci = axT + (size_t)i * N;
    int j;
    for (j = i + 1; j < L; j++) {
      const uint8_t *cj = axT + (size_t)j * N;
      int n[25] = {0};
      long long r[K4] = {0}, c[K4] = {0}, nA = 0, sq = 0;
      int x, y, t;
      for (t = 0; t < N; t++) n[ci[t] * 5 + cj[t]]++;
      for (x = 0; x < K4; x++)
        for (y = 0; y < K4; y++)
          if (is_allowed(x, y, allow)) { nA += n[x * 5 + y]; r[x] += n[x * 5 + y]; c[y] += n[x * 5 + y]; }
      for (x = 0; x < K4; x++) sq += r[x] * r[x] + c[x] * c[x];
      {
        double cij = (double)(nA * nA - sq / 2), qij = (double)(N - nA);
        qij /= N;
        cij /= (N > 1) ? (double)N * ((double)N - 1.0) : 1.0;
        cij *= 2.0;
        COV[(int64_t)i * L + j] = COV[(int64_t)j * L + i] = cij - 1.0 * qij;
      }
    }
  }
  for (i = 0; i < L - 1; i++) {
    int j;
    for (j = i + 1; j < L; j++) {
      const double v = COV[(int64_t)i * L + j];
      if (v < minmax[0]) minmax[0] = v;
      if (v > minmax[1]) minmax[1] = v;
    }
  }
  free(axT);
  return 0;
}

/* corr_CalculateRAF, src/correlators.c:876-933, unweighted, O(N^2) per pair;
 * beyond 10^11 sequence-pair x column-pair steps the count form above */
int
orc_raf(const uint8_t *ax, int N, int L, const double *allow, double *COV, double *minmax)
{
  int i, j, s1, s2;
  if (0.5 * (double)N * N * 0.5 * (double)L * L > 1e11) return orc_raf_counts(ax, N, L, allow, COV, minmax);
  cov_reset(L, COV, minmax);
  for (i = 0; i < L - 1; i++)
    for (j = i + 1; j < L; j++) {
      double cij = 0.0, qij = 0.0;
      for (s1 = 0; s1 < N; s1++) {
        int ai = ax[(int64_t)s1 * L + i], aj = ax[(int64_t)s1 * L + j];
        int al = is_allowed(ai, aj, allow);
        if (!al) qij += 1.0;
        for (s2 = s1 + 1; s2 < N; s2++) {
          int bi = ax[(int64_t)s2 * L + i], bj = ax[(int64_t)s2 * L + j];
          if (al && is_allowed(bi, bj, allow)) {
            if      (ai != bi && aj != bj) cij += 2.0;
            else if (ai != bi || aj != bj) cij += 1.0;
          }
        }
      }
      qij /= N;
      cij /= (N > 1) ? (double)N * ((double)N - 1.0) : 1.0;
      cij *= 2.0;
      cov_set(L, COV, minmax, i, j, cij - 1.0 * qij);
    }
  return 0;
}

/* corr_CalculateRAF's loop (src/correlators.c:876-933) for npairs listed
 * pairs (i < j) only, over the host threads: out[k] = RAF of (pi[k], pj[k]) */
void
orc_raf_pairs(const uint8_t *ax, int N, int L, const double *allow, int npairs, const int *pi, const int *pj,
              double *out)
{
  int k;
#pragma omp parallel for schedule(dynamic, 1)
  for (k = 0; k < npairs; k++) {
    const int i = pi[k], j = pj[k];
    double cij = 0.0, qij = 0.0;
    int s1, s2;
    for (s1 = 0; s1 < N; s1++) {
      int ai = ax[(int64_t)s1 * L + i], aj = ax[(int64_t)s1 * L + j];
      int al = is_allowed(ai, aj, allow);
      if (!al) { qij += 1.0; continue; }
      for (s2 = s1 + 1; s2 < N; s2++) {
        int bi = ax[(int64_t)s2 * L + i], bj = ax[(int64_t)s2 * L + j];
        if (is_allowed(bi, bj, allow)) {
          if      (ai != bi && aj != bj) cij += 2.0;
          else if (ai != bi || aj != bj) cij += 1.0;
        }
      }
    }
    qij /= N;
    cij /= (N > 1) ? (double)N * ((double)N - 1.0) : 1.0;
    cij *= 2.0;
    out[k] = cij - 1.0 * qij;
  }
}

/* corr_CalculateRAFS, src/correlators.c:935-982 */
int
orc_rafs(const uint8_t *ax, int N, int L, const double *allow, double *COV, double *minmax)
{
  double *b = malloc(sizeof(double) * (size_t)L * L);
  int i, j;
  if (!b) return 1;
  orc_raf(ax, N, L, allow, COV, minmax);
  memcpy(b, COV, sizeof(double) * (size_t)L * L);
  cov_reset(L, COV, minmax);
  for (i = 0; i < L - 1; i++)
    for (j = i + 1; j < L; j++) {
      double v = 2.0 * b[(int64_t)i * L + j];
      if (i > 0 && j < L - 1) v += b[(int64_t)(i - 1) * L + j + 1];
      if (j > 0 && i < L - 1 && i < j - 2) v += b[(int64_t)(i + 1) * L + j - 1];
      v *= 0.25;
      cov_set(L, COV, minmax, i, j, v);
    }
  free(b);
  return 0;
}

/* corr_CalculateCCF_C16, src/correlators.c:1010-1061 */
int
orc_ccf(int L, const double *pm, const double *nseff, double *COV, double *minmax)
{
  double meanp[K4];
  int i, j, x, y;
  cov_reset(L, COV, minmax);
  for (x = 0; x < K4; x++) {
    meanp[x] = 0.0;
    for (i = 0; i < L; i++)
      for (j = i + 1; j < L; j++)
        meanp[x] += nseff[(int64_t)i * L + j] * pm[i * K4 + x];
  }
  vec_norm(meanp, K4);
  for (i = 0; i < L - 1; i++)
    for (j = i + 1; j < L; j++) {
      double ne = nseff[(int64_t)i * L + j], ccf = 0.0;
      for (x = 0; x < K4; x++)
        for (y = 0; y < K4; y++) {
          double cc = (ne * pm[i * K4 + x] - meanp[x]) * (ne * pm[j * K4 + y] - meanp[y]);
          ccf += cc * cc;
        }
      cov_set(L, COV, minmax, i, j, sqrt(ccf));
    }
  return 0;
}

/* corr_CalculateCOVCorrected, src/correlators.c:1063-1157 (no shift) */
int
orc_cov_corrected(int actype, int L, double *COV, double *minmax)
{
  double *COVx = malloc(sizeof(double) * (L > 0 ? L : 1));
  double  avg = 0.0;
  double *C = malloc(sizeof(double) * (size_t)L * L);
  int     i, j;
  if (!COVx || !C) return 1;
  memcpy(C, COV, sizeof(double) * (size_t)L * L);
  for (i = 0; i < L - 1; i++)
    for (j = i + 1; j < L; j++) avg += C[(int64_t)i * L + j];
  if (L > 1) avg /= (double)L * ((double)L - 1.);
  avg *= 2.;
  for (i = 0; i < L; i++) {
    COVx[i] = 0.0;
    for (j = 0; j < L; j++) if (j != i) COVx[i] += C[(int64_t)i * L + j];
    if (L > 1) COVx[i] /= (double)L - 1.;
  }
  minmax[0] = INFINITY; minmax[1] = -INFINITY;
  for (i = 0; i < L; i++)
    for (j = 0; j < L; j++) {
      double v;
      if (i == j) continue;
      if (actype == ORC_APC) v = (avg != 0.0) ? C[(int64_t)i * L + j] - COVx[i] * COVx[j] / avg : 0.0;
      else                   v = C[(int64_t)i * L + j] - (COVx[i] + COVx[j] - avg);
      if (isnan(v)) { free(COVx); free(C); return 2; }
      COV[(int64_t)i * L + j] = v;
      if (v < minmax[0]) minmax[0] = v;
      if (v > minmax[1]) minmax[1] = v;
    }
  free(COVx); free(C);
  return 0;
}

/* the statistic of covtype and its correction, from probabilities already
 * formed for this alignment (RAF and RAFS read the alignment itself) */
static int
cov_from_probs(int covtype, int covclass, const uint8_t *ax, int N, int L, int nseqthresh, int alenthresh,
               const double *allow, const double *pp, const double *nseff, const double *ngap, const double *pm,
               double *COV, double *minmax)
{
  int base = (covtype / 3) * 3, corr = covtype % 3;   /* 0 none, 1 APC, 2 ASC */
  int status;
  if (base == ORC_RAF)       status = orc_raf (ax, N, L, allow, COV, minmax);
  else if (base == ORC_RAFS) status = orc_rafs(ax, N, L, allow, COV, minmax);
  else if (base == ORC_CCF)  status = orc_ccf(L, pm, nseff, COV, minmax);
  else status = orc_stat(base, covclass, N, L, nseqthresh, alenthresh, pp, pm, nseff, ngap, allow, COV, minmax);
  if (status) return status;
  if (corr == 1) status = orc_cov_corrected(ORC_APC, L, COV, minmax);
  if (corr == 2) status = orc_cov_corrected(ORC_ASC, L, COV, minmax);
  return status;
}

static int
needs_probs(int covtype)
{
  const int base = (covtype / 3) * 3;
  return base != ORC_RAF && base != ORC_RAFS;
}

/* cov_Calculate dispatch, src/covariation.c:63-306 (NONPARAM, no power) */
int
orc_cov_calculate(int covtype, int covclass, const uint8_t *ax, const double *wgt, int N, int L,
                  int nseqthresh, int alenthresh, const double *allow, double tol,
                  double *COV, double *minmax)
{
  double *pp = NULL, *nseff = NULL, *ngap = NULL, *pm = NULL, *ps = NULL;
  int status = 0;
  if (needs_probs(covtype)) {
    pp    = malloc(sizeof(double) * (size_t)L * L * K16);
    nseff = malloc(sizeof(double) * (size_t)L * L);
    ngap  = malloc(sizeof(double) * (size_t)L * L);
    pm    = malloc(sizeof(double) * (size_t)L * K4);
    ps    = malloc(sizeof(double) * (size_t)L * 5);
    if (!pp || !nseff || !ngap || !pm || !ps) status = 1;
    if (!status) status = orc_probs(ax, wgt, N, L, tol, pp, nseff, ngap, pm, ps);
  }
  if (!status)
    status = cov_from_probs(covtype, covclass, ax, N, L, nseqthresh, alenthresh, allow, pp, nseff, ngap, pm, COV,
                            minmax);
  free(pp); free(nseff); free(ngap); free(pm); free(ps);
  return status;
}

/* ------------------------------------------------------------------ */
/* Histograms -- Easel ESL_HISTOGRAM semantics, restated               */
/* bin b holds (bmin + b*w, bmin + (b+1)*w]                            */
/* ------------------------------------------------------------------ */
orc_hist_t *
orc_hist_create(double bmin, double bmax, double w)
{
  orc_hist_t *h = calloc(1, sizeof(orc_hist_t));
  if (!h) return NULL;
  h->bmin = bmin; h->bmax = bmax; h->w = w;
  h->nb = (int)((bmax - bmin) / w);
  if (h->nb < 1) h->nb = 1;
  h->obs = calloc(h->nb, sizeof(uint64_t));
  h->xmin = INFINITY; h->xmax = -INFINITY;
  h->imin = h->nb; h->imax = -1; h->cmin = h->nb;
  h->phi = 0.0;
  return h;
}

void
orc_hist_free(orc_hist_t *h)
{
  if (h) { free(h->obs); free(h); }
}

int
orc_hist_score2bin(const orc_hist_t *h, double x)
{
  return (int)ceil(((x - h->bmin) / h->w) - 1.0);
}

double orc_hist_lbound(const orc_hist_t *h, int b) { return h->w * b + h->bmin; }
double orc_hist_ubound(const orc_hist_t *h, int b) { return h->w * (b + 1) + h->bmin; }

/* growth rules as spelled out at src/covariation.c:1776-1808 */
int
orc_hist_add(orc_hist_t *h, double x)
{
  int b = orc_hist_score2bin(h, x), nnew, i;
  if (!isfinite(x)) return 1;
  if (b < 0) {
    uint64_t *o;
    nnew = -b * 2;
    o = calloc((size_t)h->nb + nnew, sizeof(uint64_t));
    memcpy(o + nnew, h->obs, sizeof(uint64_t) * h->nb);
    free(h->obs); h->obs = o;
    h->nb += nnew; b += nnew; h->bmin -= nnew * h->w;
    h->imin += nnew; h->cmin += nnew;
    if (h->imax > -1) h->imax += nnew;
  } else if (b >= h->nb) {
    nnew = (b - h->nb + 1) * 2;
    h->obs = realloc(h->obs, sizeof(uint64_t) * ((size_t)h->nb + nnew));
    for (i = h->nb; i < h->nb + nnew; i++) h->obs[i] = 0;
    if (h->imin == h->nb) { h->imin += nnew; h->cmin += nnew; }
    h->bmax += nnew * h->w;
    h->nb   += nnew;
  }
  h->obs[b]++;
  h->n++; h->Nc++; h->No++;
  if (b < h->imin) { h->imin = b; h->cmin = b; }
  if (b > h->imax) h->imax = b;
  if (x < h->xmin) h->xmin = x;
  if (x > h->xmax) h->xmax = x;
  return 0;
}

static void
hist_extend(orc_hist_t *h, int nb)
{ /* src/covariation.c:462-466 */
  int i;
  if (h->nb >= nb) return;
  h->obs = realloc(h->obs, sizeof(uint64_t) * nb);
  for (i = h->nb; i < nb; i++) h->obs[i] = 0;
  h->nb = nb;
}

/* cov_ranklist_Bin2Bin, src/covariation.c:2334-2362 */
static int
bin2bin(const orc_hist_t *h, int b, const orc_hist_t *nw)
{
  double x = orc_hist_lbound(h, b);
  return (int)round((x - nw->bmin) / nw->w);
}

/* null_add2cumranklist (src/R-scape.c:1564-1612) with cov_GrowRankList
 * (src/covariation.c:682-736): the cumulative null histogram. */
static orc_hist_t *
null_add(orc_hist_t *cum, const orc_hist_t *h)
{
  int b, cb;
  if (h == NULL) return cum;
  if (cum == NULL) {
    cum = orc_hist_create(h->bmin, h->bmax, h->w);
    cum->n = h->n; cum->xmin = h->xmin; cum->xmax = h->xmax; cum->imin = h->imin; cum->imax = h->imax;
  } else {
    double new_bmin = cum->bmin, bmax = (h->bmax > cum->bmax) ? h->bmax : cum->bmax;
    orc_hist_t *nw;
    if (h->bmin < cum->bmin) new_bmin -= fabs(h->bmin) * 2. * cum->w;
    nw = orc_hist_create(new_bmin, bmax, cum->w);
    nw->n = cum->n; nw->xmin = cum->xmin; nw->xmax = cum->xmax; nw->imin = cum->imin; nw->imax = cum->imax;
    nw->Nc = cum->Nc; nw->No = cum->No;
    for (b = cum->imin; b <= cum->imax; b++) {
      cb = bin2bin(cum, b, nw);
      if (cb < nw->nb) nw->obs[cb] = cum->obs[b];
    }
    orc_hist_free(cum);
    cum = nw;
    cum->n += h->n;
    if (h->xmin < cum->xmin) cum->xmin = h->xmin;
    if (h->xmax > cum->xmax) cum->xmax = h->xmax;
    if (h->imin < cum->imin) cum->imin = h->imin;
    if (h->imax > cum->imax) cum->imax = h->imax;
  }
  for (b = h->imin; b <= h->imax; b++) {
    cb = bin2bin(h, b, cum);
    if (cb < cum->nb) { cum->obs[cb] += h->obs[b]; cum->Nc += h->obs[b]; cum->No += h->obs[b]; }
  }
  return cum;
}

/* the contact predicates of the two-set test (CMAP_IsContactLocal,
 * CMAP_IsBPLocal, CMAP_IsWCLocal, lib/R-view/src/rview_contacts.c:537-574):
 * does any contact (i, j) (1-based, either order) satisfy the sample's rule */
static int
cnt_select(const orc_params_t *p, int64_t i, int64_t j)
{
  int64_t ii = (i < j) ? i : j, jj = (i < j) ? j : i;
  int h;
  for (h = 0; h < p->ncnt; h++) {
    if (p->cnt_i[h] != ii || p->cnt_j[h] != jj) continue;
    switch (p->samplesize) {
      case ORC_SAMPLE_CONTACTS: return 1;
      case ORC_SAMPLE_BP:       if (p->cnt_type[h] < ORC_STACKED) return 1; break;
      case ORC_SAMPLE_WC:       if (p->cnt_type[h] == ORC_WWc) return 1; break;
      default:                  return 0;
    }
  }
  return 0;
}

/* CMAP_GetBPTYPE (rview_contacts.c:523-535): the type of the first contact
 * (i, j), BPNONE if none */
static int
cnt_type(const orc_params_t *p, int64_t i, int64_t j)
{
  int64_t ii = (i < j) ? i : j, jj = (i < j) ? j : i;
  int h;
  for (h = 0; h < p->ncnt; h++)
    if (p->cnt_i[h] == ii && p->cnt_j[h] == jj) return p->cnt_type[h];
  return ORC_BPNONE;
}

/* cov_CreateHitList's isbp (src/covariation.c:836-841) */
static int
cnt_isbp(const orc_params_t *p, int bptype)
{
  switch (p->samplesize) {
    case ORC_SAMPLE_CONTACTS: return bptype < ORC_BPNONE;
    case ORC_SAMPLE_BP:       return bptype < ORC_STACKED;
    case ORC_SAMPLE_WC:       return bptype == ORC_WWc;
    default:                  return 0;
  }
}

/* cov_SignificantPairs_Ranking histogram part, src/covariation.c:414-457:
 * every pair not excluded by the PDB distance rule goes to ha; with
 * classes (the GIVSS run) the selected pairs go to hb, the others to ht. */
static orc_hist_t *
rank_scores(const orc_params_t *p, int L, const double *COV, double maxCOV, double bmin, double w, double tol,
            orc_hist_t **ret_hb, orc_hist_t **ret_ht)
{
  double bmax = maxCOV + 5 * w;
  orc_hist_t *h, *hb = NULL, *ht = NULL;
  int i, j;
  while (fabs(bmax - bmin) < tol) bmax += w;
  h = orc_hist_create(bmin, bmax, w);
  if (ret_hb) { hb = orc_hist_create(bmin, bmax, w); ht = orc_hist_create(bmin, bmax, w); }
  for (i = 0; i < L - 1; i++)
    for (j = i + 1; j < L; j++) {
      double v = COV[(int64_t)i * L + j], add = (v > bmin + w) ? v : bmin + w;
      if (p->msa2pdb && p->msa2pdb[i] >= 0 && p->msa2pdb[j] >= 0 && p->msa2pdb[j] - p->msa2pdb[i] < p->mind)
        continue;
      orc_hist_add(h, add);
      if (hb) orc_hist_add(cnt_select(p, i + 1, j + 1) ? hb : ht, add);
    }
  if (ret_hb) { *ret_hb = hb; *ret_ht = ht; }
  return h;
}

/* cov_histogram_pmass, src/covariation.c:2483-2505 */
static double
hist_pmass(const orc_hist_t *h, double target_pmass, double target_fracfit)
{
  int i, tp = 0, nfit = 0;
  uint64_t c = 0;
  double pmass = NAN;
  for (i = h->imax; i >= h->imin; i--) if (h->obs[i] > 0) tp++;
  for (i = h->imax; i >= h->imin; i--) {
    c += h->obs[i];
    if (h->obs[i] > 0) {
      nfit++;
      pmass = (double)c / (double)h->Nc;
      if ((double)nfit / (double)tp >= target_fracfit || pmass >= target_pmass) break;
    }
  }
  return pmass;
}

/* esl_histogram_SetTailByMass restated: the tail is the smallest top set of
 * bins holding at least pmass of the observations; phi is its lower bound. */
static double
hist_set_tail(orc_hist_t *h, double pmass)
{
  uint64_t sum = 0;
  int b;
  for (b = h->imax; b >= h->imin; b--) {
    sum += h->obs[b];
    if ((double)sum >= pmass * (double)h->n) break;
  }
  if (b < h->imin) b = h->imin;
  h->phi  = orc_hist_lbound(h, b);
  h->cmin = b;
  h->Nc   = h->n;
  h->No   = sum;
  return (double)sum / (double)h->n;
}

/* --- regularised incomplete gamma (series / Lentz continued fraction,
 *     Abramowitz & Stegun 6.5.29 and 6.5.31) --- */
static double
gamma_q(double a, double x)
{
  double lg = lgamma(a);
  if (x <= 0.0) return 1.0;
  if (x < a + 1.0) {
    double sum = 1.0 / a, del = sum, ap = a;
    int n;
    for (n = 0; n < 10000; n++) {
      ap += 1.0; del *= x / ap; sum += del;
      if (fabs(del) < fabs(sum) * 1e-16) break;
    }
    return 1.0 - sum * exp(-x + a * log(x) - lg);
  } else {
    double b = x + 1.0 - a, c = 1.0 / 1e-300, d = 1.0 / b, h = d;
    int i;
    for (i = 1; i < 10000; i++) {
      double an = -i * (i - a), del;
      b += 2.0;
      d = an * d + b; if (fabs(d) < 1e-300) d = 1e-300;
      c = b + an / c; if (fabs(c) < 1e-300) c = 1e-300;
      d = 1.0 / d; del = d * c; h *= del;
      if (fabs(del - 1.0) < 1e-16) break;
    }
    return exp(-x + a * log(x) - lg) * h;
  }
}

static double
gam_surv(double x, double mu, double lambda, double tau)
{
  if (x <= mu) return 1.0;
  return gamma_q(tau, lambda * (x - mu));
}

static double
exp_surv(double x, double mu, double lambda)
{
  if (x <= mu) return 1.0;
  return exp(-lambda * (x - mu));
}

/* binned gamma log likelihood over the tail bins [cmin, imax], mu = phi;
 * consecutive bins share their common boundary's survival value */
static double
gam_binned_nll(const orc_hist_t *h, double mu, double lambda, double tau)
{
  double nll = 0.0, s_hi = 0.0;
  int b, have = 0;
  for (b = h->cmin; b <= h->imax; b++) {
    double lo, slo, p;
    if (h->obs[b] == 0) { have = 0; continue; }
    lo  = orc_hist_lbound(h, b); if (lo < mu) lo = mu;
    slo = have ? s_hi : gam_surv(lo, mu, lambda, tau);
    s_hi = gam_surv(orc_hist_ubound(h, b), mu, lambda, tau);
    have = 1;
    p = slo - s_hi;
    if (!(p > 0.0)) p = 1e-300;
    nll -= (double)h->obs[b] * log(p);
  }
  return nll;
}

/* esl_gam_FitCompleteBinned restated: location fixed at phi, (lambda, tau)
 * by maximum likelihood over the binned tail; Nelder-Mead (1965) on
 * (log lambda, log tau) from method-of-moments start values. */
static int
fit_gamma(const orc_hist_t *h, double *ret_mu, double *ret_lambda, double *ret_tau)
{
  double mu = h->phi, m = 0.0, v = 0.0, n = 0.0;
  double S[3][2], F[3];
  int b, it, k;
  for (b = h->cmin; b <= h->imax; b++) {
    double mid = orc_hist_lbound(h, b) + 0.5 * h->w - mu;
    n += (double)h->obs[b]; m += (double)h->obs[b] * mid;
  }
  if (n <= 0) return 1;
  m /= n;
  for (b = h->cmin; b <= h->imax; b++) {
    double mid = orc_hist_lbound(h, b) + 0.5 * h->w - mu;
    v += (double)h->obs[b] * (mid - m) * (mid - m);
  }
  v /= n;
  if (!(v > 0.0) || !(m > 0.0)) { v = h->w * h->w; if (!(m > 0.0)) m = h->w; }
  S[0][0] = log(m / v); S[0][1] = log(m * m / v);
  S[1][0] = S[0][0] + 0.5; S[1][1] = S[0][1];
  S[2][0] = S[0][0];       S[2][1] = S[0][1] + 0.5;
  for (k = 0; k < 3; k++) F[k] = gam_binned_nll(h, mu, exp(S[k][0]), exp(S[k][1]));
  for (it = 0; it < 4000; it++) {
    int lo = 0, hi = 0, md;
    double c0, c1, r0, r1, fr;
    for (k = 1; k < 3; k++) { if (F[k] < F[lo]) lo = k; if (F[k] > F[hi]) hi = k; }
    md = 3 - lo - hi; if (md == lo || md == hi || md < 0 || md > 2) md = (hi == 0) ? ((lo == 1) ? 2 : 1) : ((hi == 1) ? ((lo == 0) ? 2 : 0) : ((lo == 0) ? 1 : 0));
    if (fabs(F[hi] - F[lo]) <= 1e-12 * (fabs(F[lo]) + 1e-30) &&
        fabs(S[hi][0] - S[lo][0]) < 1e-9 && fabs(S[hi][1] - S[lo][1]) < 1e-9) break;
    c0 = 0.5 * (S[lo][0] + S[md][0]); c1 = 0.5 * (S[lo][1] + S[md][1]);
    r0 = c0 + (c0 - S[hi][0]); r1 = c1 + (c1 - S[hi][1]);
    fr = gam_binned_nll(h, mu, exp(r0), exp(r1));
    if (fr < F[lo]) {
      double e0 = c0 + 2.0 * (c0 - S[hi][0]), e1 = c1 + 2.0 * (c1 - S[hi][1]);
      double fe = gam_binned_nll(h, mu, exp(e0), exp(e1));
      if (fe < fr) { S[hi][0] = e0; S[hi][1] = e1; F[hi] = fe; }
      else         { S[hi][0] = r0; S[hi][1] = r1; F[hi] = fr; }
    } else if (fr < F[md]) {
      S[hi][0] = r0; S[hi][1] = r1; F[hi] = fr;
    } else {
      double k0 = c0 + 0.5 * (S[hi][0] - c0), k1 = c1 + 0.5 * (S[hi][1] - c1);
      double fk = gam_binned_nll(h, mu, exp(k0), exp(k1));
      if (fk < F[hi]) { S[hi][0] = k0; S[hi][1] = k1; F[hi] = fk; }
      else {
        for (k = 0; k < 3; k++) if (k != lo) {
          S[k][0] = S[lo][0] + 0.5 * (S[k][0] - S[lo][0]);
          S[k][1] = S[lo][1] + 0.5 * (S[k][1] - S[lo][1]);
          F[k] = gam_binned_nll(h, mu, exp(S[k][0]), exp(S[k][1]));
        }
      }
    }
  }
  {
    int lo = 0;
    for (k = 1; k < 3; k++) if (F[k] < F[lo]) lo = k;
    *ret_mu = mu; *ret_lambda = exp(S[lo][0]); *ret_tau = exp(S[lo][1]);
  }
  return 0;
}

/* esl_exp_FitCompleteBinned restated: location phi; the binned exponential
 * is geometric in the bin index k, whose ML rate is
 * lambda = log(1 + 1/kbar) / w  (infinite if every count is in bin 0). */
static int
fit_exp(const orc_hist_t *h, double *ret_mu, double *ret_lambda)
{
  double n = 0.0, sk = 0.0;
  int b;
  for (b = h->cmin; b <= h->imax; b++) { n += (double)h->obs[b]; sk += (double)(b - h->cmin) * (double)h->obs[b]; }
  if (n <= 0) return 1;
  *ret_mu = h->phi;
  *ret_lambda = (sk > 0.0) ? log(1.0 + n / sk) / h->w : INFINITY;
  return 0;
}

/* cov_histogram_SetSurvFitTail, src/covariation.c:1676-1699 */
static double *
surv_tail(const orc_hist_t *h, double mass, int doexp, double mu, double lambda, double tau)
{
  double *sf = calloc((size_t)2 * h->nb, sizeof(double));
  int b;
  for (b = h->cmin; b < 2 * h->nb; b++) {
    double x = orc_hist_ubound(h, b);
    sf[b] = mass * (doexp ? exp_surv(x, mu, lambda) : gam_surv(x, mu, lambda, tau));
  }
  return sf;
}

/* cov2evalue, src/covariation.c:2369-2400 (returns INF instead of exit) */
static double
cov2evalue(double cov, double Nc, const orc_hist_t *h, const double *sf)
{
  int icov = orc_hist_score2bin(h, cov), i;
  uint64_t c = 0;
  if      (sf && icov >= 2 * h->nb - 1) return sf[2 * h->nb - 1] * Nc;
  else if (sf && cov >= h->phi)         return sf[icov + 1] * Nc;
  if (cov >= h->xmax) return Nc / (double)h->Nc;
  if (icov <= h->imax) {
    if (icov < h->imin) icov = h->imin;
    if (icov >= h->imax - 1) return Nc / (double)h->Nc;
    for (i = h->imax; i >= icov; i--) c += h->obs[i];
    return (double)c * Nc / (double)h->Nc;
  }
  return INFINITY;
}

/* the empirical branch's counts of cov2evalue for every bin at once:
 * suf[k] = sum of obs[imin + k .. imax] (exact integer sums, so
 * cov2evalue_suf returns exactly what cov2evalue's loop gives, in O(1) per
 * pair instead of O(bins)); NULL when imax < imin or out of memory */
static uint64_t *
cov2evalue_suffix(const orc_hist_t *h)
{
  uint64_t *suf;
  int i;
  if (h->imax < h->imin) return NULL;
  suf = malloc(sizeof(uint64_t) * (size_t)(h->imax - h->imin + 1));
  if (!suf) return NULL;
  suf[h->imax - h->imin] = h->obs[h->imax];
  for (i = h->imax - 1; i >= h->imin; i--) suf[i - h->imin] = suf[i - h->imin + 1] + h->obs[i];
  return suf;
}

/* cov2evalue with the suffix table (falls back to the loop without one) */
static double
cov2evalue_suf(double cov, double Nc, const orc_hist_t *h, const double *sf, const uint64_t *suf)
{
  int icov;
  if (!suf) return cov2evalue(cov, Nc, h, sf);
  icov = orc_hist_score2bin(h, cov);
  if      (sf && icov >= 2 * h->nb - 1) return sf[2 * h->nb - 1] * Nc;
  else if (sf && cov >= h->phi)         return sf[icov + 1] * Nc;
  if (cov >= h->xmax) return Nc / (double)h->Nc;
  if (icov <= h->imax) {
    if (icov < h->imin) icov = h->imin;
    if (icov >= h->imax - 1) return Nc / (double)h->Nc;
    return (double)suf[icov - h->imin] * Nc / (double)h->Nc;
  }
  return INFINITY;
}

/* evalue2cov, src/covariation.c:2403-2435 */
static double
evalue2cov(double thr, double Nc, const orc_hist_t *h, const double *sf)
{
  double cov = -INFINITY, eval;
  uint64_t c = 0;
  int b = h->cmin - 1, i;
  if (h->No >= 10 && sf) {
    for (b = 2 * h->nb - 1; b >= h->cmin; b--) {
      eval = sf[b] * Nc;
      if (eval >= thr) break;
    }
    cov = orc_hist_lbound(h, b);
  }
  if (b == h->cmin - 1) {
    for (i = h->imax; i >= h->imin; i--) {
      c += h->obs[i];
      eval = (double)c * Nc / (double)h->Nc;
      if (eval >= thr) break;
    }
    cov = orc_hist_ubound(h, i);
  }
  return cov;
}

/* ------------------------------------------------------------------ */
/* Null alignments: Fitch ancestors + shuffled substitutions           */
/* ------------------------------------------------------------------ */

static int
choose_member(unsigned S, uint64_t seed, uint32_t null_id, uint32_t node, uint32_t col)
{ /* tree_fitch_choose, src/msatree.c:1840-1855: uniform among members */
  int m = 0, k, x;
  for (x = 0; x < 5; x++) if (S & (1u << x)) m++;
  if (m == 1) k = 0;
  else        k = (int)(((uint64_t)rng_u32(seed, TAG_FCHOOSE, null_id, node, col) * (uint64_t)m) >> 32);
  for (x = 0; x < 5; x++) if (S & (1u << x)) { if (k == 0) return x; k--; }
  return ORC_GAP;
}

/* Tree_FitchAlgorithmAncenstral + tree_fitch_column, src/msatree.c:173-227,
 * 1700-1838; up pass tree_fitch_upwards :1877-1908 (intersection over the
 * five states, else union of residues only); down pass :1810-1833. */
int
orc_fitch(const uint8_t *ax, int N, int L, const orc_tree_t *T, uint64_t seed, uint32_t null_id,
          uint8_t *allmsa)
{
  int nn = 2 * N - 1, c, n, v;
  unsigned *S = malloc(sizeof(unsigned) * nn);
  if (!S) return 1;
  for (n = 0; n < N; n++) memcpy(allmsa + (int64_t)n * L, ax + (int64_t)n * L, L);
  for (c = 0; c < L; c++) {
    for (n = 0; n < N; n++) {
      int x = ax[(int64_t)n * L + c];
      if (x <= ORC_GAP) S[n] = 1u << x;
      else S[n] = 1u << (int)(((uint64_t)rng_u32(seed, TAG_FLEAF, null_id, (uint32_t)n, (uint32_t)c) * 5u) >> 32);
    }
    for (v = N - 2; v >= 0; v--) {
      int il = (T->left[v]  <= 0) ? -T->left[v]  : N + T->left[v];
      int ir = (T->right[v] <= 0) ? -T->right[v] : N + T->right[v];
      unsigned I = S[il] & S[ir];
      S[N + v] = I ? I : ((S[il] | S[ir]) & 0xFu);
    }
    allmsa[(int64_t)N * L + c] = (uint8_t)choose_member(S[N], seed, null_id, 0, (uint32_t)c);
    for (v = 0; v < N - 1; v++) {
      int a = allmsa[(int64_t)(N + v) * L + c];
      int ch[2] = { T->left[v], T->right[v] }, k;
      for (k = 0; k < 2; k++) if (ch[k] > 0) {
        int idx = N + ch[k];
        if (S[idx] & (1u << a)) S[idx] = 1u << a;
        allmsa[(int64_t)idx * L + c] = (uint8_t)choose_member(S[idx], seed, null_id, (uint32_t)ch[k], (uint32_t)c);
      }
    }
  }
  free(S);
  return 0;
}

/* msamanip_ShuffleTreeSubstitutions, src/msamanip.c:1449-1531: shuffle the
 * columns of the Fitch reconstruction (msamanip_ShuffleColumns :1164-1233),
 * then, branch by branch from the root, copy the shuffled parent into the
 * child and replay the branch's substitution counts (measured on the
 * unshuffled reconstruction, :1625-1636) on randomly chosen positions of the
 * shuffled parent that hold the old character (shuffle_tree_substitute_all
 * :1673-1747).  Random orders come from counter-based Feistel permutations. */
int
orc_null_msa(const uint8_t *ax, int N, int L, const orc_tree_t *T, uint64_t seed, uint32_t null_id,
             uint8_t *out_ax)
{
  int      nn = 2 * N - 1, v, c, n, k;
  uint8_t *all = malloc((size_t)nn * L), *sh = malloc((size_t)nn * L);
  uint32_t rk[6];
  if (!all || !sh) return 1;
  if (N == 1) { memcpy(out_ax, ax, L); free(all); free(sh); return 0; }
  orc_fitch(ax, N, L, T, seed, null_id, all);
  rng_round_keys(seed, TAG_COLPERM, null_id, 0, rk);
  for (c = 0; c < L; c++) {
    uint32_t src = orc_feistel_perm((uint32_t)c, (uint32_t)L, rk);
    for (n = 0; n < nn; n++) sh[(int64_t)n * L + c] = all[(int64_t)n * L + src];
  }
  for (v = 0; v < N - 1; v++) {
    int ch[2] = { T->left[v], T->right[v] };
    int pidx = N + v;
    for (k = 0; k < 2; k++) {
      int cidx = (ch[k] <= 0) ? -ch[k] : N + ch[k];
      int nsub[5][5], cum[5][6], rank[5] = { 0, 0, 0, 0, 0 }, o, d, t;
      memset(nsub, 0, sizeof(nsub));
      for (c = 0; c < L; c++) {
        int a = all[(int64_t)pidx * L + c], b = all[(int64_t)cidx * L + c];
        if (a != b && a <= ORC_GAP && b <= ORC_GAP) nsub[a][b]++;
      }
      for (o = 0; o < 5; o++) { cum[o][0] = 0; for (d = 0; d < 5; d++) cum[o][d + 1] = cum[o][d] + nsub[o][d]; }
      memcpy(sh + (int64_t)cidx * L, sh + (int64_t)pidx * L, L);
      rng_round_keys(seed, TAG_SUBST, null_id, (uint32_t)cidx, rk);
      for (t = 0; t < L; t++) {
        uint32_t p = orc_feistel_perm((uint32_t)t, (uint32_t)L, rk);
        int oc = sh[(int64_t)pidx * L + p], r;
        if (oc > ORC_GAP) continue;
        r = rank[oc]++;
        if (r < cum[oc][5]) {
          for (d = 0; d < 5; d++) if (r < cum[oc][d + 1]) break;
          sh[(int64_t)cidx * L + p] = (uint8_t)d;
        }
      }
    }
  }
  memcpy(out_ax, sh, (size_t)N * L);
  free(all); free(sh);
  return 0;
}

/* ------------------------------------------------------------------ */
/* The per-alignment path                                              */
/* ------------------------------------------------------------------ */
void
orc_params_default(orc_params_t *p)
{
  memset(p, 0, sizeof(*p));
  p->covtype = ORC_GT + 1; p->covclass = ORC_CSELECT;
  p->nseqthresh = 8; p->alenthresh = 50; p->nshuffle = -1;
  p->thresh = 0.05; p->bmin = -10.0; p->w0 = 0.05; p->hpts = 400;
  p->pmass = 0.0005; p->fracfit = 1.0; p->doexpfit = 0; p->tol = 1e-6; p->seed = 42;
  p->allow[0 * 4 + 3] = p->allow[3 * 4 + 0] = 1.0;   /* src/R-scape.c:883-887 */
  p->allow[1 * 4 + 2] = p->allow[2 * 4 + 1] = 1.0;
  p->allow[2 * 4 + 3] = p->allow[3 * 4 + 2] = 1.0;
  p->samplesize = ORC_SAMPLE_ALL;
  p->expBP = -1.0;
}

/* null_rscape (src/R-scape.c:1614-1724) with calculate_width_histo
 * (:1281-1371) and the nshuffle rule (:2449-2459), then the GIVSS run
 * (:2502, cov_SignificantPairs_Ranking and cov_CreateHitList,
 * src/covariation.c:325-530, 778-1006): the one-set test, or with
 * p->samplesize and a structure's contacts the two-set test; p->expBP as
 * --structured sets it. */
int
orc_rscape(const orc_params_t *p, const uint8_t *ax, const double *wgt, int N, int L,
           const orc_tree_t *T, double *COV_out, double *Eval_out,
           uint64_t *null_obs, int null_obs_cap,
           int *hit_i, int *hit_j, double *hit_sc, double *hit_E, double *hit_p, int hit_cap,
           orc_result_t *res)
{
  return orc_rscape_multi(p, 1, &p->covtype, ax, wgt, N, L, T, COV_out, Eval_out, null_obs, null_obs_cap, hit_i,
                          hit_j, hit_sc, hit_E, hit_p, hit_cap, res);
}

/* orc_rscape for nt statistics that share the null alignments: each
 * alignment's probabilities are formed once and every statistic is scored
 * from them (as R-scape would with one run per statistic on the same nulls).
 * Per-statistic outputs are nt consecutive blocks: COV_out / Eval_out of
 * L*L, null_obs of null_obs_cap, the hit arrays of hit_cap, res[nt]. */
int
orc_rscape_multi(const orc_params_t *p, int nt, const int *covtypes, const uint8_t *ax, const double *wgt, int N,
                 int L, const orc_tree_t *T, double *COV_out, double *Eval_out, uint64_t *null_obs,
                 int null_obs_cap, int *hit_i, int *hit_j, double *hit_sc, double *hit_E, double *hit_p,
                 int hit_cap, orc_result_t *res)
{
  const size_t LL = (size_t)L * L;
  double  *COV = malloc(sizeof(double) * LL * (nt > 0 ? nt : 1)), (*mm)[2] = malloc(sizeof(double[2]) * nt);
  uint8_t *shax = malloc((size_t)N * L);
  double  *pp = NULL, *nseff = NULL, *ngap = NULL, *pm = NULL, *ps = NULL;
  orc_hist_t **cum = calloc(nt, sizeof(orc_hist_t *));
  double  *w = malloc(sizeof(double) * nt);
  double   fracfit = p->fracfit;
  int      ns = p->nshuffle, s, t, i, j, status = 0, probs = 0;

  if (!COV || !mm || !shax || !cum || !w) { status = 1; goto DONE; }
  for (t = 0; t < nt; t++) { memset(&res[t], 0, sizeof(res[t])); w[t] = p->w0; probs |= needs_probs(covtypes[t]); }
  if (probs) {
    pp    = malloc(sizeof(double) * LL * K16);
    nseff = malloc(sizeof(double) * LL);
    ngap  = malloc(sizeof(double) * LL);
    pm    = malloc(sizeof(double) * (size_t)L * K4);
    ps    = malloc(sizeof(double) * (size_t)L * 5);
    if (!pp || !nseff || !ngap || !pm || !ps) { status = 1; goto DONE; }
  }
  if (ns < 0) {
    ns = 20;
    if ((double)N * L < 1e3) ns = 200;
    if (L < 50) ns = 200;
    if (L < 40) ns = 300;
    if (N < 4)  ns = 300;
  }
  if ((double)N * L < 1e3) fracfit = 0.3;
  for (t = 0; t < nt; t++) res[t].nshuffle = ns;

  /* the scores of one alignment for every statistic, into COV + t*LL */
#define SCORE_ALL(AX)                                                                                         \
  do {                                                                                                       \
    if (probs && (status = orc_probs((AX), wgt, N, L, p->tol, pp, nseff, ngap, pm, ps))) goto DONE;          \
    for (t = 0; t < nt; t++)                                                                                 \
      if ((status = cov_from_probs(covtypes[t], p->covclass, (AX), N, L, p->nseqthresh, p->alenthresh,       \
                                   p->allow, pp, nseff, ngap, pm, COV + t * LL, mm[t])))                     \
        goto DONE;                                                                                           \
  } while (0)

  for (s = 0; s < ns && N > 1; s++) {
    if ((status = orc_null_msa(ax, N, L, T, p->seed, (uint32_t)s, shax))) goto DONE;
    SCORE_ALL(shax);
    for (t = 0; t < nt; t++) {
      orc_hist_t *hs;
      if (s == 0) {
        double lo = (p->bmin > mm[t][0]) ? p->bmin : mm[t][0], wn;
        if (mm[t][1] <= p->bmin) { status = 5; goto DONE; }
        wn = (mm[t][1] - lo) / (double)p->hpts;
        w[t] = (w[t] < wn) ? w[t] : wn;
        if (w[t] < p->tol) w[t] = 0.0;
        res[t].null_minCOV = mm[t][0]; res[t].null_maxCOV = mm[t][1];
      }
      if (w[t] < 1e-20) continue;       /* covariation.c:348-374: no ranklist */
      hs     = rank_scores(p, L, COV + t * LL, mm[t][1], p->bmin, w[t], p->tol, NULL, NULL);
      cum[t] = null_add(cum[t], hs);
      orc_hist_free(hs);
    }
  }

  SCORE_ALL(ax);
#undef SCORE_ALL
  for (t = 0; t < nt; t++) {
    const double *C = COV + t * LL;
    orc_result_t *r = &res[t];
    orc_hist_t   *h = NULL, *cm = cum[t];
    double       *sf = NULL;
    int           nhit = 0;
    r->w = w[t];
    r->minCOV = mm[t][0]; r->maxCOV = mm[t][1];
    if (COV_out) memcpy(COV_out + t * LL, C, sizeof(double) * LL);
    if (Eval_out) for (i = 0; i < (int)LL; i++) Eval_out[t * LL + i] = INFINITY;
    if (N > 1 && w[t] >= 1e-20 && cm) {
      orc_hist_t *hb = NULL, *ht = NULL;
      uint64_t   *suf = NULL;
      double Nt, Nb;
      int64_t nh = 0;   /* hits so far (h of src/covariation.c:852) */
      h = rank_scores(p, L, C, mm[t][1], p->bmin, w[t], p->tol, &hb, &ht);
      Nt = (double)ht->Nc;
      Nb = (double)hb->Nc;
      r->Nt = ht->Nc;
      r->Nb = hb->Nc;
      hist_extend(cm, h->nb);
      r->pmass_used = hist_pmass(cm, p->pmass, fracfit);
      if (isnan(r->pmass_used)) { orc_hist_free(h); status = 6; goto DONE; }
      r->newmass = hist_set_tail(cm, r->pmass_used);
      if (p->doexpfit) {
        if (fit_exp(cm, &r->mu, &r->lambda)) { orc_hist_free(h); status = 7; goto DONE; }
        r->tau = 0.0;
      } else {
        if (fit_gamma(cm, &r->mu, &r->lambda, &r->tau)) { orc_hist_free(h); status = 7; goto DONE; }
      }
      r->fit_ok = 1;
      if (!isinf(r->lambda)) sf = surv_tail(cm, r->newmass, p->doexpfit, r->mu, r->lambda, r->tau);
      /* the thresholds of base pairs and of the other pairs (:490-500) */
      r->sc_thresh = evalue2cov(p->thresh, (hb->Nc > 0) ? (double)hb->Nc : (double)h->Nc, cm, sf);
      r->sc_nbp    = evalue2cov(p->thresh, (hb->Nc > 0) ? (double)ht->Nc : (double)h->Nc, cm, sf);
      /* cov_CreateHitList (src/covariation.c:828-870): base pairs take Nb
       * tests, the others expBP while fewer than expBP hits were listed,
       * then Nt */
      suf = cov2evalue_suffix(cm);
      for (i = 0; i < L - 1; i++)
        for (j = i + 1; j < L; j++) {
          double cov  = C[(int64_t)i * L + j];
          double pv   = cov2evalue_suf(cov, 1.0, cm, sf, suf);
          int    isbp = cnt_isbp(p, cnt_type(p, i + 1, j + 1));
          double ev   = isbp ? pv * Nb : ((double)nh < p->expBP ? pv * p->expBP : pv * Nt);
          if (Eval_out) Eval_out[t * LL + (int64_t)i * L + j] = Eval_out[t * LL + (int64_t)j * L + i] = ev;
          if (ev < p->thresh || p->thresh > 1000) {
            if (nhit < hit_cap) {
              const size_t o = (size_t)t * hit_cap + nhit;
              hit_i[o] = i; hit_j[o] = j; hit_sc[o] = cov; hit_E[o] = ev; hit_p[o] = pv;
            }
            nhit++;
            nh++;
          }
        }
      free(suf);
      orc_hist_free(hb);
      orc_hist_free(ht);
    }
    r->nhit = nhit;
    if (cm) {
      r->h_bmin = cm->bmin; r->h_w = cm->w; r->h_nb = cm->nb;
      r->h_imin = cm->imin; r->h_imax = cm->imax; r->h_cmin = cm->cmin;
      r->h_n = cm->n; r->h_Nc = cm->Nc; r->h_No = cm->No;
      r->h_xmin = cm->xmin; r->h_xmax = cm->xmax; r->h_phi = cm->phi;
      if (null_obs)
        for (i = 0; i < cm->nb && i < null_obs_cap; i++) null_obs[(size_t)t * null_obs_cap + i] = cm->obs[i];
    }
    free(sf);
    orc_hist_free(h);
  }
DONE:
  if (cum) for (t = 0; t < nt; t++) orc_hist_free(cum[t]);
  free(cum); free(w); free(COV); free(mm); free(shax);
  free(pp); free(nseff); free(ngap); free(pm); free(ps);
  return status;
}

/* ------------------------------------------------------------------ */
/* Reference-faithful timing mode: the loop nest of corr_NaivePP ->    */
/* mutual_naive_ppij (per-pair column gathers from the row-major       */
/* alignment, src/correlators.c:1716-1760) followed by the GT C16 cell */
/* loop (:376-388), for the pairs of rows [i0, i1).                    */
/* ------------------------------------------------------------------ */
double
orc_faithful_rows(const uint8_t *ax, const double *wgt, int N, int L, int i0, int i1,
                  int nthreads, double *checksum)
{
  double  total = 0.0;
  double *pm = malloc(sizeof(double) * (size_t)L * K4);
  int     i, x, s;
  long long npairs = 0;
  for (i = 0; i < L; i++) {
    double *m = pm + (int64_t)i * K4;
    for (x = 0; x < K4; x++) m[x] = 1e-5;
    for (s = 0; s < N; s++) { int r = ax[(int64_t)s * L + i]; if (r < 4) m[r] += wgt[s]; }
    vec_norm(m, K4);
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+:total, npairs)
#endif
  for (i = i0; i < i1; i++) {
    int j;
    for (j = i + 1; j < L; j++) {
      int   *coli = malloc(sizeof(int) * N), *colj = malloc(sizeof(int) * N);
      double p[K16], ne = 0.0, ng = 0.0, gt = 0.0;
      int    ss, xx, y;
      for (xx = 0; xx < K16; xx++) p[xx] = 1e-10;
      for (ss = 0; ss < N; ss++) { coli[ss] = ax[(int64_t)ss * L + i]; colj[ss] = ax[(int64_t)ss * L + j]; }
      for (ss = 0; ss < N; ss++) {
        int ri = coli[ss], rj = colj[ss];
        if (ri < 4 && rj < 4) { ne += wgt[ss]; p[ri * K4 + rj] += wgt[ss]; }
        else                  { ng += wgt[ss]; }
      }
      vec_norm(p, K16);
      for (xx = 0; xx < K4; xx++)
        for (y = 0; y < K4; y++) {
          double exp = ne * pm[i * K4 + xx] * pm[j * K4 + y];
          double obs = ne * p[xx * K4 + y];
          gt += (exp > 0. && obs > 0.) ? obs * log(obs / exp) : 0.0;
        }
      total += 2.0 * gt + 1e-30 * ng;
      npairs++;
      free(coli); free(colj);
    }
  }
  free(pm);
  if (checksum) *checksum = total;
  return (double)npairs;
}

/* Reference-faithful RAF timing mode: corr_CalculateRAF's O(N^2) loop
 * (src/correlators.c:897-925) on the row-major alignment for the first
 * npairs pairs of the triangle. */
double
orc_faithful_raf(const uint8_t *ax, int N, int L, int npairs, int nthreads, double *checksum)
{
  double total = 0.0;
  int k;
  int  *pi = malloc(sizeof(int) * (npairs > 0 ? npairs : 1)), *pj = malloc(sizeof(int) * (npairs > 0 ? npairs : 1));
  int  i = 0, j = 1, n = 0;
  double allow[16] = {0, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 1, 1, 0, 1, 0};
  while (n < npairs && i < L - 1) { pi[n] = i; pj[n] = j; n++; if (++j >= L) { i++; j = i + 1; } }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+:total)
#endif
  for (k = 0; k < n; k++) {
    int a = pi[k], b = pj[k], s1, s2;
    double cij = 0.0, qij = 0.0;
    for (s1 = 0; s1 < N; s1++) {
      int ai = ax[(int64_t)s1 * L + a], aj = ax[(int64_t)s1 * L + b];
      int al = is_allowed(ai, aj, allow);
      if (!al) qij += 1.0;
      for (s2 = s1 + 1; s2 < N; s2++) {
        int bi = ax[(int64_t)s2 * L + a], bj = ax[(int64_t)s2 * L + b];
        if (al && is_allowed(bi, bj, allow)) {
          if      (ai != bi && aj != bj) cij += 2.0;
          else if (ai != bi || aj != bj) cij += 1.0;
        }
      }
    }
    total += 2.0 * cij / ((double)N * (N - 1.0)) - qij / N;
  }
  free(pi); free(pj);
  if (checksum) *checksum = total;
  return (double)n;
}

/* ------------------------------------------------------------------ */
/* P(t) alignment simulator                                            */
/* ------------------------------------------------------------------ */

/* P = exp(t Q) (esl_dmx_Exp at src/ratematrix.c:208): A = t Q / 2^k with
 * the largest absolute row sum of A at most 1/2, P = sum_{m <= 18} A^m / m!,
 * then k squarings */
int
orc_sim_expm(const double *Q, int n, double t, double *P)
{
  double A[256], term[256], tmp[256], nrm = 0.0, r;
  int i, j, l, m, k = 0;
  if (n < 1 || n > 16) return 1;
  for (i = 0; i < n; i++) {
    r = 0.0;
    for (j = 0; j < n; j++) r += fabs(Q[i * n + j] * t);
    if (r > nrm) nrm = r;
  }
  while (nrm > 0.5) { nrm *= 0.5; k++; }
  for (i = 0; i < n * n; i++) A[i] = Q[i] * t / ldexp(1.0, k);
  for (i = 0; i < n * n; i++) { P[i] = (i % (n + 1) == 0) ? 1.0 : 0.0; term[i] = P[i]; }
  for (m = 1; m <= 18; m++) {
    for (i = 0; i < n; i++)
      for (j = 0; j < n; j++) {
        double s = 0.0;
        for (l = 0; l < n; l++) s += term[i * n + l] * A[l * n + j];
        tmp[i * n + j] = s / m;
      }
    for (i = 0; i < n * n; i++) { term[i] = tmp[i]; P[i] += term[i]; }
  }
  for (; k > 0; k--) {
    for (i = 0; i < n; i++)
      for (j = 0; j < n; j++) {
        double s = 0.0;
        for (l = 0; l < n; l++) s += P[i * n + l] * P[l * n + j];
        tmp[i * n + j] = s;
      }
    for (i = 0; i < n * n; i++) P[i] = tmp[i];
  }
  return 0;
}

/* ratematrix_ConditionalsFromRate (src/ratematrix.c:185-233): a time in
 * (-1e-5, 0) becomes 1e-5, a more negative one fails; times above 1e4 are
 * capped (the branch that maps 0 to 1e-4 is overwritten by the cap's else
 * branch, so time 0 gives the identity); negative entries above -1e-3 are
 * zeroed, others fail; rows are renormalised */
int
orc_sim_conditionals(const double *Q, int n, double rt, double *P)
{
  double time;
  int i, j;
  if (rt < 0.0) {
    if (rt > -1e-5) rt = 1e-5;
    else return 1;
  }
  time = (rt > 10000.0) ? 10000.0 : rt;
  if (orc_sim_expm(Q, n, time, P)) return 1;
  for (i = 0; i < n; i++) {
    double s = 0.0;
    for (j = 0; j < n; j++) {
      if (P[i * n + j] < 0.0) {
        if (fabs(P[i * n + j]) < 0.001) P[i * n + j] = 0.0;
        else return 2;
      }
    }
    for (j = 0; j < n; j++) s += P[i * n + j];
    if (!(s > 0.0)) return 2;
    for (j = 0; j < n; j++) P[i * n + j] /= s;
  }
  return 0;
}

void
orc_sim_cdf(const double *P, int n, int nrows, uint64_t *C)
{
  int i, j;
  for (i = 0; i < nrows; i++) {
    double c = 0.0;
    for (j = 0; j < n; j++) {
      c += P[i * n + j];
      if (j == n - 1 || c >= 1.0) C[i * n + j] = UINT64_MAX;
      else                        C[i * n + j] = (uint64_t)ldexp(c, 64);
    }
  }
}

/* cov_addres / cov_addpair: the first state whose running sum exceeds the
 * uniform (here the 64-bit draw U against the thresholds) */
static int
sim_draw(const uint64_t *C, int n, uint64_t U)
{
  int i;
  for (i = 0; i < n - 1; i++) if (U < C[i]) return i;
  return n - 1;
}

/* units: an unpaired column c (partner -1) or a base pair c < ct[c], in
 * column order */
static int
sim_units(int L, const int *ct, int *ua, int *ub)
{
  int c, n = 0;
  for (c = 0; c < L; c++) {
    if (ct[c] >= 0 && ct[c] < c) continue;
    ua[n] = c; ub[n] = (ct[c] > c) ? ct[c] : -1; n++;
  }
  return n;
}

/* cov_evolve_root_ungapped_tree + cov_emit_ungapped + cov_substitute
 * (src/cov_simulate.c:288-324,586-631,725-798): internal nodes in index
 * order, each child drawn from its branch's conditional on the parent's
 * state; then per leaf the gap process: a gapped column continues the run
 * with probability pext, any other column opens one with probability popen
 * (gap_rate / gap_mean, mean run length gap_mean) */
int
orc_simulate(const orc_tree_t *T, int N, int L, const int *ct, const uint64_t *C4, const uint64_t *C16,
             const uint64_t *R4, const uint64_t *R16, const uint8_t *root, double gap_rate, double gap_mean,
             uint64_t seed, uint32_t rep, uint8_t *out)
{
  int *ua = malloc(sizeof(int) * (L + 1)), *ub = malloc(sizeof(int) * (L + 1));
  uint8_t *st = NULL;
  int nu, u, v, s, n, c;
  const double popen = (gap_mean > 0.0) ? gap_rate / gap_mean : 0.0;
  const double pext = (gap_mean > 1.0) ? 1.0 - 1.0 / gap_mean : 0.0;
  if (!ua || !ub) { free(ua); free(ub); return 5; }
  nu = sim_units(L, ct, ua, ub);
  st = malloc((size_t)(N > 1 ? N - 1 : 1) * nu);
  if (!st) { free(ua); free(ub); return 5; }
  for (u = 0; u < nu; u++) {
    int x;
    if (root) {
      if (root[ua[u]] > 3 || (ub[u] >= 0 && root[ub[u]] > 3)) { free(ua); free(ub); free(st); return 11; }
      x = (ub[u] >= 0) ? root[ua[u]] * 4 + root[ub[u]] : root[ua[u]];
    } else {
      const uint64_t U = rng_u64(seed, TAG_SIMROOT, rep, 0u, (uint32_t)u);
      x = (ub[u] >= 0) ? sim_draw(R16, 16, U) : sim_draw(R4, 4, U);
    }
    st[u] = (uint8_t)x;
  }
  for (v = 0; v < N - 1; v++)
    for (s = 0; s < 2; s++) {
      const int ch = s ? T->right[v] : T->left[v];
      const int b = 2 * v + s;
      const uint32_t cid = (uint32_t)((ch <= 0) ? -ch : N + ch);
      for (u = 0; u < nu; u++) {
        const int a = st[(size_t)v * nu + u];
        const uint64_t U = rng_u64(seed, TAG_SIMSUB, rep, cid, (uint32_t)u);
        const int x = (ub[u] >= 0) ? sim_draw(C16 + ((size_t)b * 16 + a) * 16, 16, U)
                                   : sim_draw(C4 + ((size_t)b * 4 + a) * 4, 4, U);
        if (ch > 0) st[(size_t)ch * nu + u] = (uint8_t)x;
        else if (ub[u] >= 0) { out[(size_t)(-ch) * L + ua[u]] = (uint8_t)(x / 4); out[(size_t)(-ch) * L + ub[u]] = (uint8_t)(x % 4); }
        else out[(size_t)(-ch) * L + ua[u]] = (uint8_t)x;
      }
    }
  for (n = 0; n < N; n++) {
    int run = 0;
    for (c = 0; c < L; c++) {
      uint32_t key[2] = { (uint32_t)seed, (uint32_t)(seed >> 32) };
      uint32_t ctr[4] = { TAG_SIMGAP, rep, (uint32_t)n, (uint32_t)c }, o[4];
      double ue, uo;
      orc_philox4x32(key, ctr, o);
      ue = (double)o[0] * (1.0 / 4294967296.0);
      uo = (double)o[1] * (1.0 / 4294967296.0);
      if ((run && ue < pext) || uo < popen) { out[(size_t)n * L + c] = 4; run = 1; }
      else run = 0;
    }
  }
  free(ua); free(ub); free(st);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Tree_Substitutions (src/msatree.c:1423-1554) and the power lookups of */
/* power_SPAIR_Create (src/power.c:65-218)                              */
/* ------------------------------------------------------------------ */
int
orc_substitutions(const uint8_t *ax, int N, int L, const orc_tree_t *T, uint64_t seed, uint32_t null_id,
                  int includegaps, int *nsubs, int *ndouble, int *njoin)
{
  uint8_t *all = malloc((size_t)(2 * N - 1) * L);
  int i, j, v, k;
  if (!all) return 5;
  if (orc_fitch(ax, N, L, T, seed, null_id, all)) { free(all); return 1; }
  for (i = 0; i < L; i++) nsubs[i] = 0;
  for (i = 0; i < L * L; i++) { ndouble[i] = 0; njoin[i] = 0; }
  for (v = 0; v < N - 1; v++) {
    const uint8_t *p = all + (int64_t)(N + v) * L;
    for (k = 0; k < 2; k++) {
      const int ch = k ? T->right[v] : T->left[v];
      const uint8_t *c = all + (int64_t)((ch > 0) ? N + ch : -ch) * L;
      for (i = 0; i < L; i++) {
        if (includegaps) { if (c[i] != p[i]) nsubs[i]++; }
        else if (p[i] < 4 && c[i] < 4 && c[i] != p[i]) nsubs[i]++;
      }
      for (i = 0; i < L - 1; i++)
        for (j = i + 1; j < L; j++) {
          if (includegaps) {
            if (c[i] != p[i] && c[j] != p[j]) ndouble[i * L + j]++;
            if (c[i] != p[i] || c[j] != p[j]) njoin[i * L + j]++;
          } else if (p[i] < 4 && p[j] < 4 && c[i] < 4 && c[j] < 4) {
            if (c[i] != p[i] && c[j] != p[j]) ndouble[i * L + j]++;
            if (c[i] != p[i] || c[j] != p[j]) njoin[i * L + j]++;
          }
        }
    }
  }
  free(all);
  return 0;
}

double
orc_power_step(double n, int ns, const double *subs, const double *prob)
{
  double p = 0.0;
  int s;
  for (s = 0; s < ns; s++) {
    if (n > subs[s]) p = prob[s];
    else break;
  }
  return p;
}

/* ------------------------------------------------------------------------
 * Learned null: features and the network, restated in FP64 from the
 * library's own definitions (no reference counterpart).
 * ------------------------------------------------------------------------ */
static uint64_t orc_splitmix64(uint64_t x) {   /* Steele, Lea & Flood 2014 */
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

static int orc_bin16(double v, double scale) {
  const double q = v * scale;
  if (!(q >= 0.0)) return 0;
  return q >= 15.0 ? 15 : (int)q;
}

void orc_features(const uint8_t *ax, int N, int L, const double *w, double tree_len, double *feat) {
  const int NPAIR = 4096;
  double sw = 0.0, sw2 = 0.0;
  for (int s = 0; s < N; s++) { sw += w[s]; sw2 += w[s] * w[s]; }
  const double wmean = sw / N;
  double wvar = 0.0;
  for (int s = 0; s < N; s++) wvar += (w[s] - wmean) * (w[s] - wmean);
  wvar /= N;
  double *H = malloc(sizeof(double) * L), *g = malloc(sizeof(double) * L);
  double comp[4] = {0, 0, 0, 0};
  int hist[2][16];
  memset(hist, 0, sizeof(hist));
  for (int c = 0; c < L; c++) {
    double n[4] = {0, 0, 0, 0};
    for (int s = 0; s < N; s++) {
      const int x = ax[(size_t)s * L + c];
      if (x < 4) n[x] += w[s];
    }
    const double r = (n[0] + n[1]) + (n[2] + n[3]);
    double h = 0.0;
    if (r > 0.0)
      for (int x = 0; x < 4; x++)
        if (n[x] > 0.0) { const double p = n[x] / r; h -= p * log2(p); }
    H[c] = h;
    g[c] = sw > 0.0 ? fmax(0.0, (sw - r) / sw) : 0.0;
    for (int x = 0; x < 4; x++) comp[x] += n[x];
    hist[0][orc_bin16(H[c], 8.0)]++;
    hist[1][orc_bin16(g[c], 16.0)]++;
  }
  double mH = 0, mg = 0, vH = 0, vg = 0;
  for (int c = 0; c < L; c++) { mH += H[c]; mg += g[c]; }
  mH /= L; mg /= L;
  for (int c = 0; c < L; c++) { vH += (H[c] - mH) * (H[c] - mH); vg += (g[c] - mg) * (g[c] - mg); }
  vH /= L; vg /= L;
  const long long npair_all = (long long)N * (N - 1) / 2;
  const int M = npair_all < NPAIR ? (int)npair_all : NPAIR;
  double *id = malloc(sizeof(double) * (M > 0 ? M : 1));
  for (int k = 0; k < M; k++) {
    int i, j;
    if (npair_all <= NPAIR) {
      int rem = k;
      i = 0;
      while (rem >= N - 1 - i) { rem -= N - 1 - i; i++; }
      j = i + 1 + rem;
    } else {
      const uint64_t h = orc_splitmix64(0x5EED1DE7ull + (uint64_t)k);
      i = (int)((uint32_t)h % (uint32_t)N);
      j = (int)((uint32_t)(h >> 32) % (uint32_t)(N - 1));
      if (j >= i) j++;
    }
    int both = 0, same = 0;
    for (int c = 0; c < L; c++) {
      const int x = ax[(size_t)i * L + c], y = ax[(size_t)j * L + c];
      if (x < 4 && y < 4) { both++; same += (x == y); }
    }
    id[k] = both ? (double)same / (double)both : 0.0;
  }
  double mid = 0, vid = 0;
  for (int k = 0; k < M; k++) mid += id[k];
  if (M) mid /= M;
  for (int k = 0; k < M; k++) vid += (id[k] - mid) * (id[k] - mid);
  if (M) vid /= M;
  const double rtot = (comp[0] + comp[1]) + (comp[2] + comp[3]);
  feat[0] = log((double)N);
  feat[1] = log((double)L);
  feat[2] = sw2 > 0.0 ? log(sw * sw / sw2) : 0.0;
  feat[3] = mid;
  feat[4] = tree_len;
  for (int q = 0; q < 2; q++)
    for (int b = 0; b < 16; b++) feat[5 + 16 * q + b] = (double)hist[q][b] / (double)L;
  feat[37] = sqrt(vid);
  feat[38] = mH;
  feat[39] = sqrt(vH);
  feat[40] = mg;
  feat[41] = sqrt(vg);
  feat[42] = wmean > 0.0 ? sqrt(wvar) / wmean : 0.0;
  for (int x = 0; x < 4; x++) feat[43 + x] = rtot > 0.0 ? comp[x] / rtot : 0.0;
  for (int k = 47; k < 64; k++) feat[k] = 0.0;   /* null-score summary: filled by the engine */
  free(H); free(g); free(id);
}

/* round-to-nearest-even of an FP32 value to BF16, returned as a double */
static double orc_bf16(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return (double)f;   /* inf/NaN kept */
  u += 0x7FFFu + ((u >> 16) & 1u);
  u &= 0xFFFF0000u;
  float r;
  memcpy(&r, &u, 4);
  return (double)r;
}

enum { MF = 64, MH = 256, MO = 3 };
#define OW1 0
#define OB1 (OW1 + MH * MF)
#define OW2 (OB1 + MH)
#define OB2 (OW2 + MH * MH)
#define OW3 (OB2 + MH)
#define OB3 (OW3 + MH * MH)
#define OW4 (OB3 + MH)
#define OB4 (OW4 + MO * MH)
#define ONP (OB4 + MO)

static double orc_sig(double z) { return 1.0 / (1.0 + exp(-z)); }

/* forward of one standardised row x[64]: pre-activations z[3][256],
 * activations h[3][256], outputs y[3] (standardised) */
static void orc_mlp_row(const double *W, const float *params, const double *x, double z[3][MH], double h[3][MH],
                        double *y) {
  const int off_w[3] = {OW1, OW2, OW3}, off_b[3] = {OB1, OB2, OB3};
  const double *in = x;
  int nin = MF;
  for (int l = 0; l < 3; l++) {
    for (int o = 0; o < MH; o++) {
      double a = 0.0;
      for (int i = 0; i < nin; i++) a += W[off_w[l] + o * nin + i] * in[i];
      z[l][o] = a + (double)params[off_b[l] + o];
      h[l][o] = z[l][o] * orc_sig(z[l][o]);
    }
    in = h[l];
    nin = MH;
  }
  for (int o = 0; o < MO; o++) {
    double a = 0.0;
    for (int i = 0; i < MH; i++) a += W[OW4 + o * MH + i] * h[2][i];
    y[o] = a + (double)params[OB4 + o];
  }
}

static double *orc_mlp_weights(const float *params) {
  double *W = malloc(sizeof(double) * ONP);
  for (int k = 0; k < ONP; k++) W[k] = orc_bf16(params[k]);
  return W;
}

void orc_mlp_forward(const float *params, const float *nrm, const float *X, int n, double *Y) {
  double *W = orc_mlp_weights(params);
  double x[MF], z[3][MH], h[3][MH], y[MO];
  for (int r = 0; r < n; r++) {
    for (int f = 0; f < MF; f++) x[f] = ((double)X[(size_t)r * MF + f] - nrm[f]) / nrm[MF + f];
    orc_mlp_row(W, params, x, z, h, y);
    for (int o = 0; o < MO; o++) Y[(size_t)r * MO + o] = y[o] * nrm[2 * MF + MO + o] + nrm[2 * MF + o];
  }
  free(W);
}

double orc_mlp_grad(const float *params, const float *nrm, const float *X, const float *T, int n, double *grad) {
  double *W = orc_mlp_weights(params);
  double x[MF], z[3][MH], h[3][MH], y[MO], dy[MO], d[3][MH];
  double loss = 0.0;
  const double sc = 2.0 / ((double)n * MO);
  memset(grad, 0, sizeof(double) * ONP);
  for (int r = 0; r < n; r++) {
    for (int f = 0; f < MF; f++) x[f] = ((double)X[(size_t)r * MF + f] - nrm[f]) / nrm[MF + f];
    orc_mlp_row(W, params, x, z, h, y);
    for (int o = 0; o < MO; o++) {
      const double t = ((double)T[(size_t)r * MO + o] - nrm[2 * MF + o]) / nrm[2 * MF + MO + o];
      loss += (y[o] - t) * (y[o] - t);
      dy[o] = sc * (y[o] - t);
    }
    /* layer 4 */
    for (int o = 0; o < MO; o++) {
      for (int i = 0; i < MH; i++) grad[OW4 + o * MH + i] += dy[o] * h[2][i];
      grad[OB4 + o] += dy[o];
    }
    for (int i = 0; i < MH; i++) {
      double a = 0.0;
      for (int o = 0; o < MO; o++) a += dy[o] * W[OW4 + o * MH + i];
      const double s = orc_sig(z[2][i]);
      d[2][i] = a * s * (1.0 + z[2][i] * (1.0 - s));
    }
    /* layers 3, 2, 1 */
    const int off_w[3] = {OW1, OW2, OW3}, off_b[3] = {OB1, OB2, OB3};
    for (int l = 2; l >= 0; l--) {
      const double *in = l ? h[l - 1] : x;
      const int nin = l ? MH : MF;
      for (int o = 0; o < MH; o++) {
        for (int i = 0; i < nin; i++) grad[off_w[l] + o * nin + i] += d[l][o] * in[i];
        grad[off_b[l] + o] += d[l][o];
      }
      if (l == 0) break;
      for (int i = 0; i < MH; i++) {
        double a = 0.0;
        for (int o = 0; o < MH; o++) a += d[l][o] * W[off_w[l] + o * MH + i];
        const double s = orc_sig(z[l - 1][i]);
        d[l - 1][i] = a * s * (1.0 + z[l - 1][i] * (1.0 - s));
      }
    }
  }
  free(W);
  return loss / ((double)n * MO);
}

/* ------------------------------------------------------------------ */
/* Helix aggregation, src/aggregate.c                                  */
/* ------------------------------------------------------------------ */
/* chi-square upper tail Q(df/2, x/2): esl_stats_ChiSquaredTest and
 * esl_stats_IncompleteGamma's Q, as the reference calls them
 * (src/aggregate.c:171, 228, 281) */
static double
chisq_q(double df, double x)
{
  return gamma_q(df / 2.0, x / 2.0);
}

/* esl_gam_invcdf(P, 0, 1/2, w/2) of src/aggregate.c:216 and :269: the x with
 * P(w/2, x/2) = P, the lower tail, by bisection of the regularised gamma.
 * The reference passes P = 1 - p; the same rounding of 1 - p is kept here,
 * so the upper tail inverted is q = 1 - (1 - p). */
static double
chisq_invcdf_lower(double P, double w)
{
  double q = 1.0 - P, lo = 0.0, hi = 1.0;
  int    k;
  if (q >= 1.0) return 0.0;
  if (q <= 0.0) return INFINITY;
  while (chisq_q(w, hi) > q && hi < 1e300) hi *= 2.0;
  for (k = 0; k < 2000 && hi - lo > 1e-15 * hi; k++) {
    double mid = 0.5 * (lo + hi);
    if (chisq_q(w, mid) > q) lo = mid; else hi = mid;
  }
  return 0.5 * (lo + hi);
}

/* agg_FISHER, src/aggregate.c:146-179 */
double
orc_agg_fisher(int n, const double *p)
{
  double chival = 0.0;
  int    i;
  if (n == 1) return p[0];
  for (i = 0; i < n; i++) chival += -2.0 * log(p[i]);
  return chisq_q(2.0 * n, chival);
}

/* agg_LANCASTER, src/aggregate.c:195-238, and agg_WFISHER, :250-291: the
 * weighted chi-square quantiles of the p-values summed, then the upper tail
 * with sum_i w_i degrees of freedom */
double
orc_agg_weighted(int n, const double *p, const double *w)
{
  double df = 0.0, chival = 0.0;
  int    i;
  if (n == 1) return p[0];
  for (i = 0; i < n; i++) df += w[i];
  for (i = 0; i < n; i++) chival += chisq_invcdf_lower(1.0 - p[i], w[i]);
  return chisq_q(df, chival);
}

/* agg_SIDAK, src/aggregate.c:299-322 */
double
orc_agg_sidak(int n, const double *p)
{
  double pmin = p[0];
  int    i;
  if (n == 1) return p[0];
  for (i = 1; i < n; i++) if (p[i] < pmin) pmin = p[i];
  return 1.0 - exp((double)n * log(1.0 - pmin));
}

/* extract_rm_weights_lancaster, src/aggregate.c:375-416 (AGG_SINGLE): the
 * pair's substitution count plus delta = 1 */
void
orc_agg_weights_lancaster(int n, const double *nsubs, double *w)
{
  int i;
  for (i = 0; i < n; i++) w[i] = 1.0 + nsubs[i];
}

/* extract_rm_weights_wfisher, src/aggregate.c:431-488 (AGG_SINGLE): the
 * pair's power plus epsilon = 0.01, scaled so that the weights sum to 2n */
void
orc_agg_weights_wfisher(int n, const double *power, double *w)
{
  double sum = 0.0;
  int    i;
  for (i = 0; i < n; i++) w[i] = 0.01 + power[i];
  for (i = 0; i < n; i++) sum += w[i];
  if (sum > 0.0)
    for (i = 0; i < n; i++) w[i] *= 2.0 * n / sum;
}
