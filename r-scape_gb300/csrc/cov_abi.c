/* cov_abi.c -- the reference-named entry points of R-scape's covariation
 * path (src/correlators.h:445-482, src/covariation.h:27-60) on top of the
 * GB300 engine.
 *
 * State: every struct mutual_s owns one engine context for its nseq x alen
 * shape (created on first use).  corr_NaivePP / corr_Probs upload the
 * alignment and count on the device; the corr_Calculate* functions score
 * the alignment last uploaded for that object and fill mi->COV (both
 * triangles, diagonal -inf, as corr_ReuseCOV leaves it); the corrections,
 * histograms and E-values run on the device from mi->COV.  The host keeps the
 * reference's arrays (pp, nseff, ngap, pm, ps, COV, Eval) so that callers
 * reading them (power_SPAIR_AddMI, CaCoFold, dot plots) see the same layout.
 * With mi->device_resident set, pp/nseff/ngap and the score matrix stay on
 * the device instead: no L x L array crosses the bus between
 * corr_Calculate* and cov_CreateHitList, and corr_SyncHost copies COV back on
 * request.  For a shuffled alignment (mi->ishuffled, which R-scape sets
 * through corr_Create / corr_Reuse for its null alignments,
 * src/R-scape.c:2432,2574) pp/nseff/ngap and the score matrix stay on the
 * device in both modes: R-scape reads those arrays only for the given
 * alignment (power_SPAIR_AddMI in GIVSS mode, src/covariation.c:260-263;
 * CaCoFold outside RANSS mode, src/R-scape.c:2682) and takes from a null
 * its ranklist and minCOV/maxCOV (src/R-scape.c:1353-1360,1685-1690), so
 * the host arrays are neither cleared nor filled for a null and keep what
 * the last given alignment left there.
 *
 * Scope: the one-set test (SAMPLE_ALL; every pair tested alike) and the
 * two-set test (R-scape -s: the given structure's contacts against the other
 * pairs), --structured (expBP) and the PDB distance rule (msa2pdb).  Files the
 * reference writes from cov_CreateHitList (.cov, .sorted.cov, .power) and
 * helix aggregation belong to its output layer and are not produced here.
 */
#include "covgpu.h"
#include "rscape_cov.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define XFAIL(code, errbuf, ...)                                \
  do {                                                          \
    if (errbuf) snprintf((errbuf), 256, __VA_ARGS__);           \
    return (code);                                              \
  } while (0)

typedef struct {
  covgpu_ctx *ctx;
  int         have_msa;
  int         have_counts;
  int         cov_on_dev;  /* the device alone holds mi's current scores (device-resident mode, or a
                            * shuffled alignment) */
  double     *wgt;        /* weights of the uploaded alignment */
  void       *pinned[5];  /* host arrays page-locked for the copies (pp, nseff, ngap, COV, Eval) */
  uint8_t    *axbuf;      /* the alignment's codes, contiguous, page-locked once (axpinned) */
  int         axpinned;
} gpu_state;

/* host-array mode copies pp (L^2 16 doubles), nseff, ngap, COV and Eval
 * between host and device for every alignment: page-locked once per
 * mutual_s, those copies run at the link's DMA rate */
static void
pin_host(struct mutual_s *mi, gpu_state *g)
{
  const size_t LL = (size_t)mi->alen * (size_t)mi->alen;
  void  *p[5] = {mi->pp[0][0], mi->nseff[0], mi->ngap[0], mi->COV->mx[0], mi->Eval->mx[0]};
  size_t n[5] = {LL * 16 * sizeof(double), LL * sizeof(double), LL * sizeof(double), LL * sizeof(double),
                 LL * sizeof(double)};
  int k;
  if (mi->device_resident) return;
  for (k = 0; k < 5; k++)
    if (!g->pinned[k] && covgpu_host_pin(p[k], n[k]) == 0) g->pinned[k] = p[k];
}

static void
unpin_host(gpu_state *g)
{
  int k;
  for (k = 0; k < 5; k++) { covgpu_host_unpin(g->pinned[k]); g->pinned[k] = NULL; }
}

/* whether pp, nseff, ngap and the scores of the current alignment go to the
 * host arrays: not in device-resident mode, and not for a shuffled (null)
 * alignment, whose pair probabilities and score matrix R-scape never reads
 * (it takes the null's ranklist and minCOV / maxCOV) */
static int
probs_on_host(const struct mutual_s *mi)
{
  return !mi->device_resident && !mi->ishuffled;
}

/* the score matrix to hand to the engine: NULL = the device's own copy */
static const double *
cov_src(struct mutual_s *mi)
{
  gpu_state *g = (gpu_state *)mi->gpu;
  return (g && g->cov_on_dev) ? NULL : mi->COV->mx[0];
}

static gpu_state *
gpu(struct mutual_s *mi, char *errbuf)
{
  gpu_state *g = (gpu_state *)mi->gpu;
  if (!g) {
    g = (gpu_state *)calloc(1, sizeof(gpu_state));
    if (!g) return NULL;
    mi->gpu = g;
  }
  if (!g->ctx) {
    int st = covgpu_create(&g->ctx, 0, (int)mi->nseq, (int)mi->alen, 1, 0);
    if (st) {
      if (errbuf) snprintf(errbuf, 256, "GPU context: %s", g->ctx ? covgpu_errmsg(g->ctx) : "cannot create");
      covgpu_destroy(g->ctx);
      g->ctx = NULL;
      return NULL;
    }
  }
  pin_host(mi, g);
  return g;
}

static ESL_DMATRIX *
dmx_create(int n, int m)
{
  ESL_DMATRIX *D = (ESL_DMATRIX *)calloc(1, sizeof(ESL_DMATRIX));
  int i;
  if (!D) return NULL;
  D->n = n; D->m = m;
  D->mx = (double **)malloc(sizeof(double *) * (n > 0 ? n : 1));
  if (!D->mx) { free(D); return NULL; }
  D->mx[0] = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * (m > 0 ? m : 1));
  if (!D->mx[0]) { free(D->mx); free(D); return NULL; }
  for (i = 1; i < n; i++) D->mx[i] = D->mx[0] + (size_t)i * m;
  return D;
}

static void
dmx_destroy(ESL_DMATRIX *D)
{
  if (D) { free(D->mx[0]); free(D->mx); free(D); }
}

static void
dmx_set(ESL_DMATRIX *D, double v)
{
  const int64_t n = (int64_t)D->n * D->m;
  int64_t k;
#pragma omp parallel for schedule(static)
  for (k = 0; k < n; k++) D->mx[0][k] = v;
}

/* zero n doubles with the host's threads (corr_Reuse clears L^2 16 of them) */
static void
zero_doubles(double *p, size_t n)
{
  const int64_t nc = (int64_t)((n + 65535) / 65536);
  int64_t c;
#pragma omp parallel for schedule(static)
  for (c = 0; c < nc; c++) {
    const size_t a = (size_t)c * 65536, b = (a + 65536 < n) ? a + 65536 : n;
    memset(p + a, 0, sizeof(double) * (b - a));
  }
}

/* ---------------------------------------------------------------------- */
/* corr_Create / Reuse / ReuseCOV / Destroy  (src/correlators.c:1160-1297) */
/* ---------------------------------------------------------------------- */
struct mutual_s *
corr_Create(int64_t alen, int64_t nseq, int ishuffled, int nseqthresh, int alenthresh, const ESL_ALPHABET *abc,
            COVCLASS covclass)
{
  struct mutual_s *mi;
  int64_t i, j, L = alen;
  if (alen < 1 || nseq < 1) return NULL;
  mi = (struct mutual_s *)calloc(1, sizeof(struct mutual_s));
  if (!mi) return NULL;
  mi->alen = alen; mi->nseq = nseq; mi->nseqthresh = nseqthresh; mi->alenthresh = alenthresh;
  mi->ishuffled = ishuffled; mi->abc = abc;
  mi->pp    = (double ***)malloc(sizeof(double **) * L);
  mi->nseff = (double **)malloc(sizeof(double *) * L);
  mi->ngap  = (double **)malloc(sizeof(double *) * L);
  mi->pm    = (double **)malloc(sizeof(double *) * L);
  mi->ps    = (double **)malloc(sizeof(double *) * L);
  if (!mi->pp || !mi->nseff || !mi->ngap || !mi->pm || !mi->ps) { corr_Destroy(mi); return NULL; }
  mi->pp[0]    = (double **)malloc(sizeof(double *) * L * L);
  mi->nseff[0] = (double *)calloc((size_t)L * L, sizeof(double));
  mi->ngap[0]  = (double *)calloc((size_t)L * L, sizeof(double));
  mi->pm[0]    = (double *)calloc((size_t)L * 4, sizeof(double));
  mi->ps[0]    = (double *)calloc((size_t)L * 5, sizeof(double));
  if (!mi->pp[0] || !mi->nseff[0] || !mi->ngap[0] || !mi->pm[0] || !mi->ps[0]) { corr_Destroy(mi); return NULL; }
  mi->pp[0][0] = (double *)calloc((size_t)L * L * 16, sizeof(double));
  if (!mi->pp[0][0]) { corr_Destroy(mi); return NULL; }
  for (i = 0; i < L; i++) {
    mi->pp[i]    = mi->pp[0] + i * L;
    mi->nseff[i] = mi->nseff[0] + i * L;
    mi->ngap[i]  = mi->ngap[0] + i * L;
    mi->pm[i]    = mi->pm[0] + i * 4;
    mi->ps[i]    = mi->ps[0] + i * 5;
    for (j = 0; j < L; j++) mi->pp[i][j] = mi->pp[0][0] + (i * L + j) * 16;
  }
  mi->COV  = dmx_create((int)L, (int)L);
  mi->Eval = dmx_create((int)L, (int)L);
  if (!mi->COV || !mi->Eval) { corr_Destroy(mi); return NULL; }
  /* the reference's initial values, whatever the object is made for */
  dmx_set(mi->COV, -INFINITY);
  dmx_set(mi->Eval, INFINITY);
  corr_ReuseCOV(mi, COVNONE, covclass);
  return mi;
}

int
corr_ReuseCOV(struct mutual_s *mi, COVTYPE mitype, COVCLASS miclass)
{
  mi->type = mitype;
  mi->class_ = miclass;
  /* device-resident mode or a shuffled alignment: the host matrices are
   * written only by corr_SyncHost */
  if (mi->COV && probs_on_host(mi))  dmx_set(mi->COV, -INFINITY);
  if (mi->Eval && probs_on_host(mi)) dmx_set(mi->Eval, INFINITY);
  mi->besthreshCOV = -INFINITY;
  mi->minCOV = INFINITY;
  mi->maxCOV = -INFINITY;
  return eslOK;
}

int
corr_Reuse(struct mutual_s *mi, int ishuffled, COVTYPE mitype, COVCLASS miclass)
{
  const size_t L = (size_t)mi->alen;
  mi->ishuffled = ishuffled;
  if (probs_on_host(mi)) {   /* else pp, nseff, ngap live on the device */
    zero_doubles(mi->pp[0][0], L * L * 16);
    zero_doubles(mi->nseff[0], L * L);
    zero_doubles(mi->ngap[0], L * L);
  }
  memset(mi->pm[0], 0, sizeof(double) * L * 4);
  memset(mi->ps[0], 0, sizeof(double) * L * 5);
  return corr_ReuseCOV(mi, mitype, miclass);
}

void
corr_Destroy(struct mutual_s *mi)
{
  gpu_state *g;
  if (!mi) return;
  g = (gpu_state *)mi->gpu;
  if (g) {
    unpin_host(g);
    if (g->axpinned) covgpu_host_unpin(g->axbuf);
    covgpu_destroy(g->ctx);
    free(g->axbuf);
    free(g->wgt);
    free(g);
  }
  if (mi->pp)    { if (mi->pp[0]) free(mi->pp[0][0]); free(mi->pp[0]); free(mi->pp); }
  if (mi->nseff) { free(mi->nseff[0]); free(mi->nseff); }
  if (mi->ngap)  { free(mi->ngap[0]); free(mi->ngap); }
  if (mi->pm)    { free(mi->pm[0]); free(mi->pm); }
  if (mi->ps)    { free(mi->ps[0]); free(mi->ps); }
  dmx_destroy(mi->COV);
  dmx_destroy(mi->Eval);
  free(mi);
}

/* ---------------------------------------------------------------------- */
/* probabilities                                                            */
/* ---------------------------------------------------------------------- */
static int
upload_msa(struct mutual_s *mi, ESL_MSA *msa, char *errbuf)
{
  gpu_state *g;
  uint8_t   *ax;
  int64_t    s, L = msa->alen;
  int        st;
  if (msa->nseq != mi->nseq || msa->alen != mi->alen)
    XFAIL(eslEINVAL, errbuf, "alignment %d x %lld does not match mutual_s %lld x %lld", msa->nseq,
          (long long)msa->alen, (long long)mi->nseq, (long long)mi->alen);
  if (!(g = gpu(mi, errbuf))) return eslFAIL;
  /* one staging buffer per mutual_s, page-locked, for every alignment it
   * scores (R-scape's nulls and the alignment itself) */
  if (!g->axbuf) {
    g->axbuf = (uint8_t *)malloc((size_t)msa->nseq * L);
    if (!g->axbuf) XFAIL(eslEMEM, errbuf, "out of memory");
    g->axpinned = covgpu_host_pin(g->axbuf, (size_t)msa->nseq * L) == 0;
  }
  ax = g->axbuf;
  for (s = 0; s < msa->nseq; s++) memcpy(ax + s * L, msa->ax[s] + 1, (size_t)L);
  st = covgpu_set_alignment(g->ctx, 0, ax);
  if (st) XFAIL(eslFAIL, errbuf, "%s", covgpu_errmsg(g->ctx));
  /* the weights again only when they changed (R-scape's nulls carry the
   * alignment's) */
  {
    int same = g->wgt != NULL;
    for (s = 0; same && s < msa->nseq; s++) same = g->wgt[s] == (msa->wgt ? msa->wgt[s] : 1.0);
    if (!same) {
      free(g->wgt);
      g->wgt = (double *)malloc(sizeof(double) * msa->nseq);
      if (!g->wgt) XFAIL(eslEMEM, errbuf, "out of memory");
      for (s = 0; s < msa->nseq; s++) g->wgt[s] = msa->wgt ? msa->wgt[s] : 1.0;
      if ((st = covgpu_set_weights(g->ctx, g->wgt))) {
        /* forget them, so the next alignment uploads its weights again */
        free(g->wgt);
        g->wgt = NULL;
        XFAIL(eslFAIL, errbuf, "%s", covgpu_errmsg(g->ctx));
      }
    }
  }
  g->have_msa = 1;
  g->have_counts = 0;
  return eslOK;
}

static const double ALLOW_DEFAULT[16] = {0, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 1, 1, 0, 1, 0};

static void
allow16(const ESL_DMATRIX *allowpair, double *a)
{
  int x, y;
  for (x = 0; x < 4; x++)
    for (y = 0; y < 4; y++) a[x * 4 + y] = allowpair ? allowpair->mx[x][y] : ALLOW_DEFAULT[x * 4 + y];
}

/* covgpu_score on the tensor cores, or on SIMT where the tensor path does
 * not serve the shape (status 12) */
static int
score_dev(gpu_state *g, struct mutual_s *mi, int covtype, int cls, const double *allow, double *mm)
{
  /* the counts of corr_Probs on the same alignment are reused */
  int st = covgpu_score_reuse(g->ctx, 0, 1, 1, &covtype, cls, mi->nseqthresh, mi->alenthresh, allow,
                              COVGPU_COUNT_TENSOR, mm);
  if (st == 12)
    st = covgpu_score_reuse(g->ctx, 0, 1, 1, &covtype, cls, mi->nseqthresh, mi->alenthresh, allow,
                            COVGPU_COUNT_SIMT, mm);
  return st;
}

static int
count_on_device(struct mutual_s *mi, char *errbuf)
{
  gpu_state *g = (gpu_state *)mi->gpu;
  int st;
  if (!g || !g->have_msa) XFAIL(eslFAIL, errbuf, "no alignment uploaded (call corr_Probs first)");
  st = score_dev(g, mi, GT, C16, ALLOW_DEFAULT, NULL);
  if (st) XFAIL(eslFAIL, errbuf, "%s", covgpu_errmsg(g->ctx));
  g->have_counts = 1;
  return eslOK;
}

/* corr_NaivePP, src/correlators.c:1300-1317 */
int
corr_NaivePP(ESL_RANDOMNESS *r, ESL_MSA *msa, struct mutual_s *mi, double tol, int verbose, char *errbuf)
{
  gpu_state *g;
  int st;
  (void)r; (void)tol; (void)verbose;
  if ((st = upload_msa(mi, msa, errbuf))) return st;
  if ((st = count_on_device(mi, errbuf))) return st;
  g = (gpu_state *)mi->gpu;
  if (!probs_on_host(mi)) return eslOK;   /* pp, nseff, ngap stay on the device */
  if (covgpu_get_probs(g->ctx, 0, g->wgt, mi->pp[0][0], mi->nseff[0], mi->ngap[0], NULL, NULL))
    XFAIL(eslFAIL, errbuf, "%s", covgpu_errmsg(g->ctx));
  return eslOK;
}

/* corr_NaivePS, src/correlators.c:1319-1335 */
int
corr_NaivePS(ESL_RANDOMNESS *r, ESL_MSA *msa, struct mutual_s *mi, double tol, int verbose, char *errbuf)
{
  gpu_state *g = (gpu_state *)mi->gpu;
  int st;
  (void)r; (void)tol; (void)verbose;
  if (!g || !g->have_counts) {
    if ((st = upload_msa(mi, msa, errbuf))) return st;
    if ((st = count_on_device(mi, errbuf))) return st;
    g = (gpu_state *)mi->gpu;
  }
  if (covgpu_get_probs(g->ctx, 0, g->wgt, NULL, NULL, NULL, NULL, mi->ps[0]))
    XFAIL(eslFAIL, errbuf, "%s", covgpu_errmsg(g->ctx));
  return eslOK;
}

/* corr_Marginals, src/correlators.c:1337-1375: the marginals of the counts
 * of the last corr_NaivePP on the device */
int
corr_Marginals(struct mutual_s *mi, double tol, int verbose, char *errbuf)
{
  gpu_state *g = (gpu_state *)mi->gpu;
  int64_t i;
  (void)verbose;
  if (!g || !g->have_counts) XFAIL(eslFAIL, errbuf, "corr_Marginals: no counts on the device (call corr_NaivePP)");
  if (covgpu_get_probs(g->ctx, 0, g->wgt, NULL, NULL, NULL, mi->pm[0], NULL))
    XFAIL(eslFAIL, errbuf, "%s", covgpu_errmsg(g->ctx));
  for (i = 0; i < mi->alen; i++) {
    double s = mi->pm[i][0] + mi->pm[i][1] + mi->pm[i][2] + mi->pm[i][3];
    if (fabs(s - 1.0) > tol) XFAIL(eslFAIL, errbuf, "pm[%lld] does not sum to one", (long long)i);
  }
  return eslOK;
}

static int
validate_vec(const double *v, int n, double tol)
{
  double s = 0.0;
  int k;
  for (k = 0; k < n; k++) { if (!(v[k] >= 0.0 && v[k] <= 1.0 + tol)) return 1; s += v[k]; }
  return fabs(s - 1.0) > tol;
}

/* corr_ValidateProbs, src/correlators.c:1499-1545; the pair probabilities
 * are checked on the device when they stay there (device-resident mode, or
 * a shuffled alignment) */
int
corr_ValidateProbs(struct mutual_s *mi, double tol, int verbose, char *errbuf)
{
  int64_t i, j;
  gpu_state *g = (gpu_state *)mi->gpu;
  (void)verbose;
  if (!probs_on_host(mi) && g && g->have_counts) {
    if (covgpu_validate_probs(g->ctx, tol)) XFAIL(eslFAIL, errbuf, "pp validation failed");
  } else {
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(| : bad) private(j)
    for (i = 0; i < mi->alen - 1; i++)
      for (j = i + 1; j < mi->alen && !bad; j++)
        if (validate_vec(mi->pp[i][j], 16, tol)) bad = 1;
    if (bad) XFAIL(eslFAIL, errbuf, "pp validation failed");
  }
  for (i = 0; i < mi->alen; i++) {
    if (validate_vec(mi->pm[i], 4, tol)) XFAIL(eslFAIL, errbuf, "pm validation failed");
    if (validate_vec(mi->ps[i], 5, tol)) XFAIL(eslFAIL, errbuf, "ps validation failed");
  }
  return eslOK;
}

/* corr_Probs, src/correlators.c:1423-1496 (NONPARAM / POTTS counting) */
int
corr_Probs(ESL_RANDOMNESS *r, ESL_MSA *msa, ESL_TREE *T, void *ribosum, struct mutual_s *mi, METHOD method,
           double tol, int verbose, char *errbuf)
{
  int st;
  (void)T; (void)ribosum;
  if (method == AKMAEV) XFAIL(eslFAIL, errbuf, "the AKMAEV pair probabilities are not provided by this library");
  if ((st = corr_NaivePP(r, msa, mi, tol, verbose, errbuf))) return st;
  if ((st = corr_NaivePS(r, msa, mi, tol, verbose, errbuf))) return st;
  if ((st = corr_Marginals(mi, tol, verbose, errbuf))) return st;
  return corr_ValidateProbs(mi, tol, verbose, errbuf);
}

/* ---------------------------------------------------------------------- */
/* statistics                                                               */
/* ---------------------------------------------------------------------- */
static int
score_into_cov(struct mutual_s *mi, int covtype, int cls, const ESL_DMATRIX *allowpair, char *errbuf)
{
  gpu_state *g = (gpu_state *)mi->gpu;
  double a[16], mm[2];
  int st;
  if (!g || !g->have_msa) XFAIL(eslFAIL, errbuf, "no alignment on the device (call corr_Probs first)");
  allow16(allowpair, a);
  st = score_dev(g, mi, covtype, cls, a, mm);
  if (st) XFAIL(eslFAIL, errbuf, "%s", covgpu_errmsg(g->ctx));
  g->cov_on_dev = !probs_on_host(mi);
  if (probs_on_host(mi) && covgpu_get_cov(g->ctx, 0, 0, mi->COV->mx[0]))
    XFAIL(eslFAIL, errbuf, "%s", covgpu_errmsg(g->ctx));
  g->have_counts = 1;
  mi->type = (COVTYPE)covtype;
  mi->minCOV = mm[0];
  mi->maxCOV = mm[1];
  return eslOK;
}

static int
resolve_class(struct mutual_s *mi, COVCLASS c)
{
  if (c == CSELECT) return (mi->nseq <= mi->nseqthresh || mi->alen <= mi->alenthresh) ? C2 : C16;
  return (int)c;
}

#define STAT_FAMILY(NAME, BASE)                                                                             \
  int corr_Calculate##NAME##_C16(struct mutual_s *mi, int verbose, char *errbuf) {                         \
    (void)verbose;                                                                                         \
    mi->class_ = C16;                                                                                      \
    return score_into_cov(mi, BASE, C16, NULL, errbuf);                                                    \
  }                                                                                                        \
  int corr_Calculate##NAME##_C2(struct mutual_s *mi, ESL_DMATRIX *allowpair, int verbose, char *errbuf) {  \
    (void)verbose;                                                                                         \
    mi->class_ = C2;                                                                                       \
    return score_into_cov(mi, BASE, C2, allowpair, errbuf);                                                \
  }                                                                                                        \
  int corr_Calculate##NAME(COVCLASS covclass, struct data_s *data) {                                       \
    struct mutual_s *mi = data->mi;                                                                        \
    int cls = resolve_class(mi, covclass);                                                                 \
    if (cls == CWC) XFAIL(eslFAIL, data->errbuf, "corr_Calculate" #NAME "() CWC not implemented\n");       \
    mi->class_ = covclass;                                                                                 \
    return score_into_cov(mi, BASE, cls, data->allowpair, data->errbuf);                                   \
  }

/* CHI :49-181, OMES :184-314, MI :493-614, MIr :617-745, MIg :748-874 */
STAT_FAMILY(CHI, CHI)
STAT_FAMILY(OMES, OMES)
STAT_FAMILY(MI, MI)
STAT_FAMILY(MIr, MIr)
STAT_FAMILY(MIg, MIg)

/* GT :316-490, with the CWC form */
int
corr_CalculateGT_C16(struct mutual_s *mi, int verbose, char *errbuf)
{
  (void)verbose;
  mi->class_ = C16;
  return score_into_cov(mi, GT, C16, NULL, errbuf);
}

int
corr_CalculateGT_C2(struct mutual_s *mi, ESL_DMATRIX *allowpair, int verbose, char *errbuf)
{
  (void)verbose;
  mi->class_ = C2;
  return score_into_cov(mi, GT, C2, allowpair, errbuf);
}

int
corr_CalculateGT_CWC(struct mutual_s *mi, ESL_DMATRIX *allowpair, int verbose, char *errbuf)
{
  (void)verbose;
  mi->class_ = C16;
  return score_into_cov(mi, GT, CWC, allowpair, errbuf);
}

int
corr_CalculateGT(COVCLASS covclass, struct data_s *data)
{
  struct mutual_s *mi = data->mi;
  int cls = resolve_class(mi, covclass);
  mi->class_ = covclass;
  return score_into_cov(mi, GT, cls, data->allowpair, data->errbuf);
}

/* RAF :876-933, RAFS :935-982: unweighted, from the given alignment */
int
corr_CalculateRAF(COVCLASS covclass, struct data_s *data, ESL_MSA *msa)
{
  int st;
  (void)covclass;
  if ((st = upload_msa(data->mi, msa, data->errbuf))) return st;
  data->mi->class_ = C2;
  return score_into_cov(data->mi, RAF, C2, data->allowpair, data->errbuf);
}

int
corr_CalculateRAFS(COVCLASS covclass, struct data_s *data, ESL_MSA *msa)
{
  int st;
  (void)covclass;
  if ((st = upload_msa(data->mi, msa, data->errbuf))) return st;
  data->mi->class_ = C2;
  return score_into_cov(data->mi, RAFS, C2, data->allowpair, data->errbuf);
}

/* CCF :984-1061 */
int
corr_CalculateCCF_C16(struct mutual_s *mi, int verbose, char *errbuf)
{
  (void)verbose;
  mi->class_ = C16;
  return score_into_cov(mi, CCF, C16, NULL, errbuf);
}

int
corr_CalculateCCF(COVCLASS covclass, struct data_s *data)
{
  (void)covclass;
  return corr_CalculateCCF_C16(data->mi, data->verbose, data->errbuf);
}

/* corr_CalculateCOVCorrected, src/correlators.c:1063-1157 */
int
corr_CalculateCOVCorrected(ACTYPE actype, struct data_s *data, int shiftnonneg)
{
  struct mutual_s *mi = data->mi;
  gpu_state *g = gpu(mi, data->errbuf);
  double mm[2];
  int64_t i, j, L = mi->alen;
  int base;
  if (!g) return eslFAIL;
  if (actype != APC && actype != ASC) XFAIL(eslFAIL, data->errbuf, "wrong correction type\n");
  if (mi->type >= PTFp) XFAIL(eslFAIL, data->errbuf, "wrong COVTYPE");
  base = ((int)mi->type / 3) * 3;
  {
    const double *src = cov_src(mi);
    if (covgpu_correct(g->ctx, src, (int)actype, src ? mi->COV->mx[0] : NULL, mm))
      XFAIL(eslFAIL, data->errbuf, "bad covariation: %s", covgpu_errmsg(g->ctx));
  }
  mi->type = (COVTYPE)(base + (actype == APC ? 1 : 2));
  mi->minCOV = mm[0];
  mi->maxCOV = mm[1];
  if (shiftnonneg) {
    /* shifted on the host, which then holds the scores */
    if (corr_SyncHost(mi, data->errbuf)) return eslFAIL;
    g->cov_on_dev = 0;
    for (i = 0; i < L; i++)
      for (j = 0; j < L; j++)
        if (i != j) mi->COV->mx[i][j] -= mi->minCOV;
  }
  return eslOK;
}

/* the device's score matrix into mi->COV, when the device alone holds it
 * (device-resident mode, or a shuffled alignment's scores) */
int
corr_SyncHost(struct mutual_s *mi, char *errbuf)
{
  gpu_state *g = (gpu_state *)mi->gpu;
  if (!g || !g->cov_on_dev) return eslOK;
  if (covgpu_get_cov(g->ctx, 0, 0, mi->COV->mx[0])) XFAIL(eslFAIL, errbuf, "%s", covgpu_errmsg(g->ctx));
  return eslOK;
}

/* corr_PostOrderPP (src/correlators.c, the Akmaev pair probabilities on a
 * tree) is outside this library */
int
corr_PostOrderPP(ESL_MSA *msa, ESL_TREE *T, void *ribosum, struct mutual_s *mi, double tol, int verbose,
                 char *errbuf)
{
  (void)msa; (void)T; (void)ribosum; (void)mi; (void)tol; (void)verbose;
  XFAIL(eslFAIL, errbuf, "corr_PostOrderPP: the AKMAEV pair probabilities are not provided by this library");
}

/* corr_COVTYPEString / corr_String2COVTYPE, src/correlators.c:1562-1662 */
static const char *COVNAMES[] = {"CHI", "CHIp", "CHIa", "GT", "GTp", "GTa", "MI", "MIp", "MIa", "MIr",
                                 "MIrp", "MIra", "MIg", "MIgp", "MIga", "OMES", "OMESp", "OMESa", "RAF", "RAFp",
                                 "RAFa", "RAFS", "RAFSp", "RAFSa", "CCF", "CCFp", "CCFa", "PTFp", "PTAp", "PTDp"};

int
corr_COVTYPEString(char **ret_covtype, COVTYPE type, char *errbuf)
{
  size_t n;
  if ((int)type < 0 || (int)type >= COVNONE) XFAIL(eslFAIL, errbuf, "wrong COVTYPE");
  n = strlen(COVNAMES[type]) + 1;
  *ret_covtype = (char *)malloc(n);
  if (!*ret_covtype) XFAIL(eslEMEM, errbuf, "out of memory");
  memcpy(*ret_covtype, COVNAMES[type], n);
  return eslOK;
}

int
corr_String2COVTYPE(char *covtype, COVTYPE *ret_type, char *errbuf)
{
  int k;
  for (k = 0; k < COVNONE; k++)
    if (covtype && strcmp(covtype, COVNAMES[k]) == 0) { *ret_type = (COVTYPE)k; return eslOK; }
  XFAIL(eslFAIL, errbuf, "wrong COVTYPE %s", covtype ? covtype : "(null)");
}

/* ---------------------------------------------------------------------- */
/* cov_Calculate and the ranking                                            */
/* ---------------------------------------------------------------------- */

/* cov_Calculate, src/covariation.c:63-306 */
int
cov_Calculate(struct data_s *data, ESL_MSA *msa, RANKLIST **ret_ranklist, HITLIST **ret_hitlist,
              RMLIST **ret_rmlist, int analyze)
{
  struct mutual_s *mi = data->mi;
  COVCLASS covclass = mi->class_;
  int base, corr, st;
  if ((int)data->covtype >= PTFp) XFAIL(eslFAIL, data->errbuf, "wrong covariation type\n");
  base = ((int)data->covtype / 3) * 3;
  corr = (int)data->covtype % 3;
  if (base != RAF && base != RAFS) {
    if ((st = corr_Probs(data->r, msa, NULL, NULL, mi, data->covmethod, data->tol, data->verbose, data->errbuf)))
      return st;
  }
  switch (base) {
    case CHI:  st = corr_CalculateCHI(covclass, data); break;
    case GT:   st = corr_CalculateGT(covclass, data); break;
    case MI:   st = corr_CalculateMI(covclass, data); break;
    case MIr:  st = corr_CalculateMIr(covclass, data); break;
    case MIg:  st = corr_CalculateMIg(covclass, data); break;
    case OMES: st = corr_CalculateOMES(covclass, data); break;
    case RAF:  st = corr_CalculateRAF(covclass, data, msa); break;
    case RAFS: st = corr_CalculateRAFS(covclass, data, msa); break;
    case CCF:  st = corr_CalculateCCF(covclass, data); break;
    default:   XFAIL(eslFAIL, data->errbuf, "wrong covariation type\n");
  }
  if (st) return st;
  if (corr == 1 && (st = corr_CalculateCOVCorrected(APC, data, 0))) return st;
  if (corr == 2 && (st = corr_CalculateCOVCorrected(ASC, data, 0))) return st;
  if (ret_rmlist) *ret_rmlist = NULL;
  if (analyze) return cov_SignificantPairs_Ranking(data, ret_ranklist, ret_hitlist, ret_rmlist);
  if (ret_ranklist) *ret_ranklist = NULL;
  if (ret_hitlist) *ret_hitlist = NULL;
  return eslOK;
}

/* histogram of the pair scores of mi->COV on the device, into h (nb bins) */
static int
rank_into(struct mutual_s *mi, ESL_HISTOGRAM *h, char *errbuf)
{
  gpu_state *g = (gpu_state *)mi->gpu;
  int64_t i, j, L = mi->alen;
  int b;
  double lo = h->bmin + h->w, xmin = INFINITY, xmax = -INFINITY;
  const double *src;
  if (!g) XFAIL(eslFAIL, errbuf, "no device context");
  src = cov_src(mi);
  if (covgpu_hist_full(g->ctx, src, h->bmin, h->w, h->nb, h->obs))
    XFAIL(eslFAIL, errbuf, "%s", covgpu_errmsg(g->ctx));
  if (!src) {
    /* the binned values are max(COV, lo): their range follows from the scores' */
    xmin = (mi->minCOV > lo) ? mi->minCOV : lo;
    xmax = (mi->maxCOV > lo) ? mi->maxCOV : lo;
  } else {
    /* over the host threads (a minimum and a maximum do not depend on the order) */
#pragma omp parallel for schedule(dynamic, 16) reduction(min : xmin) reduction(max : xmax) private(j)
    for (i = 0; i < L - 1; i++)
      for (j = i + 1; j < L; j++) {
        double v = mi->COV->mx[i][j];
        double add = (v > lo) ? v : lo;
        if (add < xmin) xmin = add;
        if (add > xmax) xmax = add;
      }
  }
  h->n = h->Nc = h->No = (uint64_t)(L * (L - 1) / 2);
  h->xmin = xmin; h->xmax = xmax;
  h->imin = h->nb; h->imax = -1;
  for (b = 0; b < h->nb; b++)
    if (h->obs[b]) { if (b < h->imin) h->imin = b; if (b > h->imax) h->imax = b; }
  h->cmin = h->imin;
  return eslOK;
}

/* pair (i, j), i < j (0-based), in the scan order of the reference's loops */
static int64_t
scan_index(int64_t i, int64_t j, int64_t L)
{
  return i * (2 * L - i - 1) / 2 + (j - i - 1);
}

/* does contact type t count as a base pair for the sample (the predicates
 * of lib/R-view/src/rview_contacts.c:537-574 and cov_CreateHitList's isbp,
 * src/covariation.c:836-841) */
static int
sample_takes(SAMPLESIZE ss, int t)
{
  switch (ss) {
    case SAMPLE_CONTACTS: return t < BPNONE;
    case SAMPLE_BP:       return t < STACKED;
    case SAMPLE_WC:       return t == WWc;
    default:              return 0;
  }
}

/* the structure's contacts over the L(L-1)/2 pairs (either output may be
 * NULL): sel, bit n set when any contact of pair n satisfies the sample's
 * rule (CMAP_Is*Local, the ranking's classes); first[n], the type of the
 * first contact of pair n, BPNONE for none (CMAP_GetBPTYPE,
 * rview_contacts.c:523-535).  A contact matches pair (i, j) only as
 * cnt.i = i + 1 < cnt.j = j + 1, as the reference compares them. */
static int
contact_maps(const CLIST *cl, SAMPLESIZE ss, int64_t L, uint32_t **ret_sel, uint8_t **ret_first)
{
  int64_t P = L * (L - 1) / 2, n;
  uint32_t *sel = NULL;
  uint8_t *first = NULL, *seen = NULL;
  int h;
  if (ret_sel) {
    sel = (uint32_t *)calloc((size_t)((P + 31) / 32) + 1, sizeof(uint32_t));
    if (!sel) return eslEMEM;
  }
  first = (uint8_t *)malloc((size_t)(P > 0 ? P : 1));
  seen  = (uint8_t *)calloc((size_t)(P > 0 ? P : 1), 1);
  if (!first || !seen) { free(sel); free(first); free(seen); return eslEMEM; }
  memset(first, BPNONE, (size_t)(P > 0 ? P : 1));
  for (h = 0; cl && h < cl->ncnt; h++) {
    const CNT *c = &cl->cnt[h];
    if (c->i < 1 || c->j > L || c->i >= c->j) continue;
    n = scan_index(c->i - 1, c->j - 1, L);
    if (!seen[n]) { seen[n] = 1; first[n] = (uint8_t)c->bptype; }
    if (sel && sample_takes(ss, (int)c->bptype)) sel[n >> 5] |= 1u << (n & 31);
  }
  free(seen);
  if (ret_sel) *ret_sel = sel;
  if (ret_first) *ret_first = first; else free(first);
  return eslOK;
}

/* the ranking on the host (src/covariation.c:420-457), for the two-set
 * classes or the PDB distance rule: every pair not excluded goes to ha and,
 * with classes, to hb (sel) or ht */
static int
rank_host(struct data_s *data, RANKLIST *rl, int classes)
{
  struct mutual_s *mi = data->mi;
  const int64_t L = mi->alen;
  const int mind = data->clist ? data->clist->mind : 0;
  uint32_t *sel = NULL;
  int64_t i, j, n = 0;
  if (corr_SyncHost(mi, data->errbuf)) return eslFAIL;
  if (classes && contact_maps(data->clist, data->samplesize, L, &sel, NULL)) XFAIL(eslEMEM, data->errbuf, "out of memory");
  for (i = 0; i < L - 1; i++)
    for (j = i + 1; j < L; j++, n++) {
      double add;
      if (data->msa2pdb && data->msa2pdb[i] >= 0 && data->msa2pdb[j] >= 0 && data->msa2pdb[j] - data->msa2pdb[i] < mind)
        continue;
      add = mi->COV->mx[i][j];
      if (add < data->bmin + data->w) add = data->bmin + data->w;
      if (covh_Add(rl->ha, add) != eslOK ||
          (classes && covh_Add(((sel[n >> 5] >> (n & 31)) & 1u) ? rl->hb : rl->ht, add) != eslOK)) {
        free(sel);
        XFAIL(eslFAIL, data->errbuf, "histogram add failed");
      }
    }
  free(sel);
  return eslOK;
}

/* cov_SignificantPairs_Ranking, src/covariation.c:325-530 */
int
cov_SignificantPairs_Ranking(struct data_s *data, RANKLIST **ret_ranklist, HITLIST **ret_hitlist,
                             RMLIST **ret_rmlist)
{
  struct mutual_s *mi = data->mi;
  RANKLIST *ranklist;
  HITLIST  *hitlist = NULL;
  double    bmax, pmass, newmass;
  int       st, classes;
  if (ret_rmlist) *ret_rmlist = NULL;
  if (ret_ranklist) *ret_ranklist = NULL;
  if (ret_hitlist) *ret_hitlist = NULL;
  if ((data->nseq > 1 && data->w < 1e-20) || data->nseq == 1) {   /* :348-412 */
    if (data->thresh) { data->thresh->sc_bp = INFINITY; data->thresh->sc_nbp = INFINITY; }
    return eslOK;
  }
  bmax = mi->maxCOV + 5 * data->w;
  while (fabs(bmax - data->bmin) < data->tol) bmax += data->w;
  ranklist = cov_CreateRankList(bmax, data->bmin, data->w);
  if (!ranklist) XFAIL(eslEMEM, data->errbuf, "out of memory");
  classes = (data->mode == GIVSS || data->mode == FOLDSS) && data->samplesize != SAMPLE_ALL;
  if (classes || data->msa2pdb) {
    /* the two-set classes or the PDB rule: ha (and hb, ht) on the host */
    if ((st = rank_host(data, ranklist, classes))) { cov_FreeRankList(ranklist); return st; }
  } else if ((st = rank_into(mi, ranklist->ha, data->errbuf))) {
    cov_FreeRankList(ranklist);
    return st;
  }
  if ((data->mode == GIVSS || data->mode == FOLDSS) && !classes) {   /* SAMPLE_ALL: every pair goes to ht */
    ESL_HISTOGRAM *ht = ranklist->ht, *ha = ranklist->ha;
    if (ht->nb < ha->nb) {
      uint64_t *o = (uint64_t *)realloc(ht->obs, sizeof(uint64_t) * ha->nb);
      if (!o) { cov_FreeRankList(ranklist); XFAIL(eslEMEM, data->errbuf, "out of memory"); }
      ht->obs = o;
    }
    memcpy(ht->obs, ha->obs, sizeof(uint64_t) * ha->nb);
    ht->nb = ha->nb; ht->bmin = ha->bmin; ht->bmax = ha->bmax;
    ht->n = ha->n; ht->Nc = ha->Nc; ht->No = ha->No; ht->xmin = ha->xmin; ht->xmax = ha->xmax;
    ht->imin = ha->imin; ht->imax = ha->imax; ht->cmin = ha->cmin;
  }
  if (data->ranklist_null && data->mode == GIVSS) {
    ESL_HISTOGRAM *hn = data->ranklist_null->ha;
    if (hn->nb < ranklist->ha->nb) {   /* :462-466 */
      int b;
      hn->obs = (uint64_t *)realloc(hn->obs, sizeof(uint64_t) * ranklist->ha->nb);
      for (b = hn->nb; b < ranklist->ha->nb; b++) hn->obs[b] = 0;
      hn->nb = ranklist->ha->nb;
    }
    pmass = covh_pmass(hn, data->pmass, data->fracfit);
    if (isnan(pmass)) { cov_FreeRankList(ranklist); XFAIL(eslFAIL, data->errbuf, "bad Null histogram fit, pmass is nan."); }
    free(data->ranklist_null->survfit);
    data->ranklist_null->survfit = NULL;
    if (data->doexpfit)
      st = cov_NullFitExponential(hn, &data->ranklist_null->survfit, pmass, &newmass, &data->mu, &data->lambda,
                                  data->verbose, data->errbuf);
    else
      st = cov_NullFitGamma(hn, &data->ranklist_null->survfit, pmass, &newmass, &data->mu, &data->lambda, &data->tau,
                            data->verbose, data->errbuf);
    if (st) { cov_FreeRankList(ranklist); return st; }
  }
  if (data->mode == GIVSS && data->thresh) {   /* :490-500 */
    const int two = ranklist->hb->Nc > 0;
    const double Nb = (double)(two ? ranklist->hb->Nc : ranklist->ha->Nc);
    const double Nn = (double)(two ? ranklist->ht->Nc : ranklist->ha->Nc);
    data->thresh->sc_bp = data->ranklist_null
                              ? covh_evalue2cov(data->thresh->val, Nb, data->ranklist_null->ha, data->ranklist_null->survfit)
                              : INFINITY;
    data->thresh->sc_nbp = data->ranklist_null
                               ? covh_evalue2cov(data->thresh->val, Nn, data->ranklist_null->ha, data->ranklist_null->survfit)
                               : INFINITY;
  }
  if (data->mode == GIVSS) {
    if ((st = cov_CreateHitList(data, mi, ranklist, &hitlist, NULL, NULL, NULL))) {
      cov_FreeRankList(ranklist);
      return st;
    }
  }
  if (ret_ranklist) *ret_ranklist = ranklist; else cov_FreeRankList(ranklist);
  if (ret_hitlist) *ret_hitlist = hitlist; else cov_FreeHitList(hitlist);
  return eslOK;
}

/* cov_CreateHitList, src/covariation.c:778-1006: E = p Nb for the pairs the
 * structure's first contact makes base pairs (two-set test), else p expBP
 * while fewer than expBP hits were listed (--structured), else p Nt */
int
cov_CreateHitList(struct data_s *data, struct mutual_s *mi, RANKLIST *ranklist, HITLIST **ret_hitlist,
                  RMLIST **ret_rmlist, char *covtype, char *threshtype)
{
  gpu_state  *g = (gpu_state *)mi->gpu;
  HITLIST    *hl;
  covgpu_hit *hits = NULL;
  int64_t     P = mi->alen * (mi->alen - 1) / 2;
  int         nhit = 0, cap, k, st;
  double      thresh = data->thresh ? data->thresh->val : 0.05;
  uint32_t   *bpmask = NULL;
  uint8_t    *first = NULL;
  (void)covtype; (void)threshtype;
  if (ret_rmlist) *ret_rmlist = NULL;
  /* the first contact's type of every pair (the hits' bptype) and, in the
   * two-set test, the base pairs */
  if (data->clist && data->clist->ncnt > 0) {
    if (contact_maps(data->clist, data->samplesize, mi->alen, NULL, &first)) XFAIL(eslEMEM, data->errbuf, "out of memory");
    if (data->samplesize != SAMPLE_ALL) {
      int64_t n;
      bpmask = (uint32_t *)calloc((size_t)((P + 31) / 32) + 1, sizeof(uint32_t));
      if (!bpmask) { free(first); XFAIL(eslEMEM, data->errbuf, "out of memory"); }
      for (n = 0; n < P; n++)
        if (sample_takes(data->samplesize, first[n])) bpmask[n >> 5] |= 1u << (n & 31);
    }
  }
  hl = (HITLIST *)calloc(1, sizeof(HITLIST));
  if (!hl) { free(first); free(bpmask); XFAIL(eslEMEM, data->errbuf, "out of memory"); }
  hl->Nt = (int64_t)ranklist->ht->Nc;
  hl->Nb = (int64_t)ranklist->hb->Nc;
  if (!data->ranklist_null) {   /* naive: every pair with E = 0 */
    if (corr_SyncHost(mi, data->errbuf)) { free(hl); free(first); free(bpmask); return eslFAIL; }
    dmx_set(mi->Eval, INFINITY);
    cap = (thresh > 0.0) ? (int)P : 0;
    hl->hit = (HIT *)calloc(cap > 0 ? cap : 1, sizeof(HIT));
    for (k = 0; k < cap; k++) {
      int64_t i = 0, rem = k;
      while (rem >= mi->alen - 1 - i) { rem -= mi->alen - 1 - i; i++; }
      hl->hit[k].i = i; hl->hit[k].j = i + 1 + rem;
      hl->hit[k].sc = mi->COV->mx[i][i + 1 + rem];
      hl->hit[k].bptype = first ? first[k] : BPNONE;
    }
    hl->nhit = cap;
  } else {
    if (!g) { free(hl); free(first); free(bpmask); XFAIL(eslFAIL, data->errbuf, "no device context"); }
    cap = (int)((P < (1 << 22)) ? P : (1 << 22));
    hits = (covgpu_hit *)malloc(sizeof(covgpu_hit) * (cap > 0 ? cap : 1));
    {
      const double *src = cov_src(mi);
      /* device-resident: neither COV nor Eval comes to the host */
      st = covgpu_evalue_sets(g->ctx, src, data->ranklist_null->ha, data->ranklist_null->survfit,
                              (double)ranklist->ht->Nc, (double)ranklist->hb->Nc, data->expBP, bpmask,
                              (thresh > MAX_EVAL) ? 2.0 * MAX_EVAL : thresh, src ? mi->Eval->mx[0] : NULL, hits,
                              cap, &nhit);
    }
    if (st) { free(hits); free(hl); free(first); free(bpmask); XFAIL(eslFAIL, data->errbuf, "%s", covgpu_errmsg(g->ctx)); }
    if (nhit > cap) nhit = cap;
    hl->hit = (HIT *)calloc(nhit > 0 ? nhit : 1, sizeof(HIT));
    for (k = 0; k < nhit; k++) {
      hl->hit[k].i = hits[k].i; hl->hit[k].j = hits[k].j;
      hl->hit[k].sc = hits[k].sc; hl->hit[k].Eval = hits[k].E; hl->hit[k].pval = hits[k].pval;
      hl->hit[k].bptype = first ? first[scan_index(hits[k].i, hits[k].j, mi->alen)] : BPNONE;
    }
    hl->nhit = nhit;
    free(hits);
  }
  free(first);
  free(bpmask);
  hl->srthit = (HIT **)malloc(sizeof(HIT *) * (hl->nhit > 0 ? hl->nhit : 1));
  for (k = 0; k < hl->nhit; k++) hl->srthit[k] = &hl->hit[k];
  *ret_hitlist = hl;
  return eslOK;
}

/* cov_THRESHTYPEString, src/covariation.c:309-323 */
int
cov_THRESHTYPEString(char **ret_threshtype, THRESHTYPE type, char *errbuf)
{
  if (type != Eval) XFAIL(eslFAIL, errbuf, "wrong THRESHTYPE");
  *ret_threshtype = (char *)malloc(5);
  if (!*ret_threshtype) XFAIL(eslEMEM, errbuf, "out of memory");
  memcpy(*ret_threshtype, "Eval", 5);
  return eslOK;
}

/* cov_SignificantPairs_ZScore, src/covariation.c:1531-1582: for every base
 * pair (i, ct[i+1]-1) of a 1-based ct, the mean and deviation of the other
 * scores of rows i and ct[i+1]-1 and the pair's z-score against the
 * partner row, printed as the reference prints them (its min of the two
 * z-scores takes the partner's twice) */
int
cov_SignificantPairs_ZScore(struct mutual_s *mi, int *msamap, int firstpos, int *ct, int verbose, char *errbuf)
{
  const int64_t L = mi->alen;
  int64_t i, j, k;
  (void)verbose;
  if (corr_SyncHost(mi, errbuf)) return eslFAIL;
  for (i = 0; i < L; i++) {
    if (ct[i + 1] > 0 && ct[i + 1] > i + 1) {
      const int64_t ip = ct[i + 1] - 1;
      double avgi = 0.0, stdi = 0.0, avgj = 0.0, stdj = 0.0, zi, zj;
      for (j = 0; j < L; j++) {
        if (j != ip) {
          if (j != i) { avgi += mi->COV->mx[i][j]; stdi += mi->COV->mx[i][j] * mi->COV->mx[i][j]; }
        } else {
          avgj = 0.0; stdj = 0.0;
          for (k = 0; k < L; k++)
            if (k != j && k != i) { avgj += mi->COV->mx[j][k]; stdj += mi->COV->mx[j][k] * mi->COV->mx[j][k]; }
          avgj /= (L - 2);
          stdj /= (L - 2);
          stdj -= avgj * avgj;
          stdj = sqrt(stdj);
        }
      }
      avgi /= (L - 2);
      stdi /= (L - 2);
      stdi -= avgi * avgi;
      stdi = sqrt(stdi);
      zi = (mi->COV->mx[i][ip] - avgi) / stdi;
      zj = (mi->COV->mx[i][ip] - avgj) / stdj;
      (void)zi;
      printf("[%d][%d] %f | %f | %f %f | %f %f\n", msamap[i] + firstpos, msamap[ip] + firstpos, zj, mi->COV->mx[i][ip],
             avgi, stdi, avgj, stdj);
    }
  }
  return eslOK;
}

/* cov_WriteHistogram, src/covariation.c:1869-1915: the survival curves of
 * the alignment's base pairs, its other pairs and the null (with its fit)
 * into covhisfile; the gnuplot figures are not drawn */
int
cov_WriteHistogram(struct data_s *data, char *gnuplot, char *covhisfile, char *covqqfile, SAMPLESIZE samplesize,
                   RANKLIST *ranklist, char *title)
{
  FILE *fp;
  int st = eslOK;
  (void)gnuplot; (void)covqqfile; (void)samplesize; (void)title;
  if (ranklist == NULL || covhisfile == NULL) return eslOK;
  if ((fp = fopen(covhisfile, "w")) == NULL) XFAIL(eslFAIL, data->errbuf, "could not open covhisfile %s\n", covhisfile);
  if (cov_histogram_PlotSurvival(fp, ranklist->hb, NULL) ||
      cov_histogram_PlotSurvival(fp, ranklist->ht, NULL) ||
      (data->ranklist_null &&
       cov_histogram_PlotSurvival(fp, data->ranklist_null->ha, data->ranklist_null->survfit)))
    st = eslFAIL;
  fclose(fp);
  if (st) XFAIL(eslFAIL, data->errbuf, "histogram survival plot write failed");
  return eslOK;
}

/* cov_CreateFOLDHitList (src/covariation.c:1009, the hit list of a
 * CaCoFold structure) is outside this library */
int
cov_CreateFOLDHitList(struct data_s *data, void *foldctlist, RANKLIST *ranklist, HITLIST *hitlist, void *r3d,
                      HITLIST **ret_foldhitlist, RMLIST **ret_foldrmlist, char *covtype, char *threshtype)
{
  (void)foldctlist; (void)ranklist; (void)hitlist; (void)r3d; (void)covtype; (void)threshtype;
  if (ret_foldhitlist) *ret_foldhitlist = NULL;
  if (ret_foldrmlist) *ret_foldrmlist = NULL;
  XFAIL(eslFAIL, data->errbuf, "cov_CreateFOLDHitList: CaCoFold's hit list is not provided by this library");
}
