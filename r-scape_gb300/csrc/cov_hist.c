/* cov_hist.c -- null-score histograms, tail fits and score <-> E-value
 * conversion of R-scape's covariation path (host side, FP64).
 *
 * R-scape keeps its score histograms in Easel ESL_HISTOGRAMs and fits their
 * tails with Easel's binned gamma/exponential fits; Easel is not part of the
 * reference tree, so the histogram rules and the fits are restated here from
 * their definitions:
 *   - bins of width w from bmin; bin b holds (bmin + b w, bmin + (b+1) w];
 *     a sample outside the allocated range grows the histogram by twice the
 *     missing number of bins (the rule spelled out at
 *     src/covariation.c:1776-1808);
 *   - the tail holding at least `pmass` of the samples, counted down from the
 *     top bin, is fitted with its lower bound phi as the location;
 *   - gamma tail: maximum likelihood of the binned counts over
 *     (lambda, tau), Nelder-Mead on (log lambda, log tau) started from
 *     moment estimates; exponential tail: the closed-form binned ML rate.
 * The per-pair conversions cov2evalue / evalue2cov and the pmass rule follow
 * src/covariation.c:2369-2435, 2483-2505.
 */
#include "rscape_cov.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

ESL_HISTOGRAM *
covh_Create(double bmin, double bmax, double w)
{
  ESL_HISTOGRAM *h = (ESL_HISTOGRAM *)calloc(1, sizeof(ESL_HISTOGRAM));
  if (!h) return NULL;
  h->bmin = bmin; h->bmax = bmax; h->w = w;
  h->nb = (int)((bmax - bmin) / w);
  if (h->nb < 1) h->nb = 1;
  h->obs = (uint64_t *)calloc((size_t)h->nb, sizeof(uint64_t));
  if (!h->obs) { free(h); return NULL; }
  h->xmin = INFINITY; h->xmax = -INFINITY;
  h->imin = h->nb; h->imax = -1; h->cmin = h->nb;
  h->phi = 0.0;
  return h;
}

void
covh_Destroy(ESL_HISTOGRAM *h)
{
  if (h) { free(h->obs); free(h); }
}

int
covh_Score2Bin(const ESL_HISTOGRAM *h, double x, int *ret_b)
{
  double b;
  if (!isfinite(x)) return eslERANGE;
  b = ceil(((x - h->bmin) / h->w) - 1.0);
  if (b < -2147483647.0 || b > 2147483647.0) return eslERANGE;
  *ret_b = (int)b;
  return eslOK;
}

double covh_Bin2LBound(const ESL_HISTOGRAM *h, int b) { return h->w * b + h->bmin; }
double covh_Bin2UBound(const ESL_HISTOGRAM *h, int b) { return h->w * (b + 1) + h->bmin; }

int
covh_Add(ESL_HISTOGRAM *h, double x)
{
  int b, nnew, i;
  if (covh_Score2Bin(h, x, &b) != eslOK) return eslERANGE;
  if (b < 0) {
    uint64_t *o;
    nnew = -b * 2;
    o = (uint64_t *)calloc((size_t)h->nb + nnew, sizeof(uint64_t));
    if (!o) return eslEMEM;
    memcpy(o + nnew, h->obs, sizeof(uint64_t) * h->nb);
    free(h->obs); h->obs = o;
    h->nb += nnew; b += nnew; h->bmin -= nnew * h->w;
    h->imin += nnew; h->cmin += nnew;
    if (h->imax > -1) h->imax += nnew;
  } else if (b >= h->nb) {
    uint64_t *o;
    nnew = (b - h->nb + 1) * 2;
    o = (uint64_t *)realloc(h->obs, sizeof(uint64_t) * ((size_t)h->nb + nnew));
    if (!o) return eslEMEM;
    h->obs = o;
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
  return eslOK;
}

/* cov_histogram_pmass, src/covariation.c:2483-2505 */
double
covh_pmass(const ESL_HISTOGRAM *h, double target_pmass, double target_fracfit)
{
  int      i, tp = 0, nfit = 0;
  uint64_t c = 0;
  double   pmass = NAN;
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

/* the tail holding >= pmass of the samples; returns the tail's mass */
double
covh_SetTailByMass(ESL_HISTOGRAM *h, double pmass)
{
  uint64_t sum = 0;
  int b;
  for (b = h->imax; b >= h->imin; b--) {
    sum += h->obs[b];
    if ((double)sum >= pmass * (double)h->n) break;
  }
  if (b < h->imin) b = h->imin;
  h->phi  = covh_Bin2LBound(h, b);
  h->cmin = b;
  h->Nc   = h->n;
  h->No   = sum;
  return (double)sum / (double)h->n;
}

/* regularised upper incomplete gamma Q(a,x): series for x < a+1, Lentz's
 * continued fraction otherwise (Abramowitz & Stegun 6.5.29, 6.5.31) */
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
    double b = x + 1.0 - a, c = 1.0 / 1e-300, d = 1.0 / b, hh = d;
    int i;
    for (i = 1; i < 10000; i++) {
      double an = -i * (i - a), del;
      b += 2.0;
      d = an * d + b; if (fabs(d) < 1e-300) d = 1e-300;
      c = b + an / c; if (fabs(c) < 1e-300) c = 1e-300;
      d = 1.0 / d; del = d * c; hh *= del;
      if (fabs(del - 1.0) < 1e-16) break;
    }
    return exp(-x + a * log(x) - lg) * hh;
  }
}

double
covh_gamma_surv(double x, void *params)
{
  const double *p = (const double *)params;   /* mu, lambda, tau */
  if (x <= p[0]) return 1.0;
  return gamma_q(p[2], p[1] * (x - p[0]));
}

double
covh_exp_surv(double x, void *params)
{
  const double *p = (const double *)params;   /* mu, lambda */
  if (x <= p[0]) return 1.0;
  return exp(-p[1] * (x - p[0]));
}

#define NLL_CHUNKS 64

/* log of the gamma probability of the bin [lo, lo + hw) when the bin is far
 * enough above mu (hw <= (lo - mu) / 16, lambda hw <= 1/2): f(x) times
 * integral_0^hw exp(g(t)) dt, x = lo - mu, g(t) = (tau-1) log(1 + t/x) - lambda t,
 * from the power series of exp(g), whose coefficients follow
 * (x + t) E' = (tau - 1 - lambda (x + t)) E:
 *   c_{k+1} = ((tau - 1 - lambda x - k) c_k - lambda c_{k-1}) / (x (k + 1)).
 * Returns 0 and leaves *ret_logp alone when the bin is too close to mu. */
static int
gam_logp_series(double lo, double hw, double mu, double lambda, double tau, double lconst, double *ret_logp)
{
  const double x = lo - mu;
  double r, s, dkm1 = 0.0, dk = 1.0, sum = 1.0;
  int k;
  if (!(x > 0.0) || hw > 0.0625 * x || lambda * hw > 0.5) return 0;
  r = hw / x; s = lambda * hw;
  for (k = 0; k < 60; k++) {
    const double dk1 = (((tau - 1.0 - k) * r - s) * dk - s * r * dkm1) / (k + 1);
    const double term = dk1 / (k + 2);
    sum += term;
    dkm1 = dk; dk = dk1;
    if (fabs(term) <= 1e-17 * fabs(sum)) break;
  }
  *ret_logp = lconst + (tau - 1.0) * log(x) - lambda * x + log(hw * sum);
  return 1;
}

/* negative log-likelihood of the tail bins [cmin, imax] under a gamma at
 * location mu: -sum_b obs_b log(S(lo_b) - S(hi_b)), the bin probability
 * taken from the series above where it applies.  The bins are summed in a
 * fixed number of chunks (in parallel when OpenMP is on) whose partial sums
 * are added in chunk order, so the result does not depend on the number of
 * threads */
static double
gam_nll(const ESL_HISTOGRAM *h, double mu, double lambda, double tau)
{
  double part[NLL_CHUNKS], prm[3], nll = 0.0;
  const int b0 = h->cmin, nbins = h->imax - h->cmin + 1;
  const double lconst = tau * log(lambda) - lgamma(tau);
  int c;
  prm[0] = mu; prm[1] = lambda; prm[2] = tau;
  if (nbins <= 0) return 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static, 1) if (nbins > 512)
#endif
  for (c = 0; c < NLL_CHUNKS; c++) {
    const int lo_b = b0 + (int)((int64_t)nbins * c / NLL_CHUNKS);
    const int hi_b = b0 + (int)((int64_t)nbins * (c + 1) / NLL_CHUNKS);
    double acc = 0.0, s_hi = 0.0;
    int b, have = 0;
    for (b = lo_b; b < hi_b; b++) {
      double lo, hi, slo, p, lp;
      if (h->obs[b] == 0) { have = 0; continue; }
      lo = covh_Bin2LBound(h, b); hi = covh_Bin2UBound(h, b);
      if (gam_logp_series(lo, hi - lo, mu, lambda, tau, lconst, &lp)) {
        acc -= (double)h->obs[b] * lp;
        have = 0;
        continue;
      }
      if (lo < mu) lo = mu;
      slo = have ? s_hi : covh_gamma_surv(lo, prm);
      s_hi = covh_gamma_surv(hi, prm);
      have = 1;
      p = slo - s_hi;
      if (!(p > 0.0)) p = 1e-300;
      acc -= (double)h->obs[b] * log(p);
    }
    part[c] = acc;
  }
  for (c = 0; c < NLL_CHUNKS; c++) nll += part[c];
  return nll;
}

/* binned ML gamma fit of the tail, location = phi */
static int
fit_gamma(const ESL_HISTOGRAM *h, double *ret_mu, double *ret_lambda, double *ret_tau)
{
  double mu = h->phi, m = 0.0, v = 0.0, n = 0.0, S[3][2], F[3];
  int b, it, k, lo;
  for (b = h->cmin; b <= h->imax; b++) {
    double mid = covh_Bin2LBound(h, b) + 0.5 * h->w - mu;
    n += (double)h->obs[b]; m += (double)h->obs[b] * mid;
  }
  if (n <= 0) return eslFAIL;
  m /= n;
  for (b = h->cmin; b <= h->imax; b++) {
    double mid = covh_Bin2LBound(h, b) + 0.5 * h->w - mu;
    v += (double)h->obs[b] * (mid - m) * (mid - m);
  }
  v /= n;
  if (!(v > 0.0) || !(m > 0.0)) { v = h->w * h->w; if (!(m > 0.0)) m = h->w; }
  /* simplex on (log lambda, log tau) */
  S[0][0] = log(m / v); S[0][1] = log(m * m / v);
  S[1][0] = S[0][0] + 0.5; S[1][1] = S[0][1];
  S[2][0] = S[0][0];       S[2][1] = S[0][1] + 0.5;
  for (k = 0; k < 3; k++) F[k] = gam_nll(h, mu, exp(S[k][0]), exp(S[k][1]));
  for (it = 0; it < 4000; it++) {
    int hi = 0, md;
    double c0, c1, r0, r1, fr;
    lo = 0;
    for (k = 1; k < 3; k++) { if (F[k] < F[lo]) lo = k; if (F[k] > F[hi]) hi = k; }
    md = 3 - lo - hi;
    if (md == lo || md == hi || md < 0 || md > 2)
      md = (hi == 0) ? ((lo == 1) ? 2 : 1) : ((hi == 1) ? ((lo == 0) ? 2 : 0) : ((lo == 0) ? 1 : 0));
    if (fabs(F[hi] - F[lo]) <= 1e-12 * (fabs(F[lo]) + 1e-30) &&
        fabs(S[hi][0] - S[lo][0]) < 1e-9 && fabs(S[hi][1] - S[lo][1]) < 1e-9) break;
    c0 = 0.5 * (S[lo][0] + S[md][0]); c1 = 0.5 * (S[lo][1] + S[md][1]);
    r0 = c0 + (c0 - S[hi][0]);       r1 = c1 + (c1 - S[hi][1]);
    fr = gam_nll(h, mu, exp(r0), exp(r1));
    if (fr < F[lo]) {
      double e0 = c0 + 2.0 * (c0 - S[hi][0]), e1 = c1 + 2.0 * (c1 - S[hi][1]);
      double fe = gam_nll(h, mu, exp(e0), exp(e1));
      if (fe < fr) { S[hi][0] = e0; S[hi][1] = e1; F[hi] = fe; }
      else         { S[hi][0] = r0; S[hi][1] = r1; F[hi] = fr; }
    } else if (fr < F[md]) {
      S[hi][0] = r0; S[hi][1] = r1; F[hi] = fr;
    } else {
      double k0 = c0 + 0.5 * (S[hi][0] - c0), k1 = c1 + 0.5 * (S[hi][1] - c1);
      double fk = gam_nll(h, mu, exp(k0), exp(k1));
      if (fk < F[hi]) { S[hi][0] = k0; S[hi][1] = k1; F[hi] = fk; }
      else {
        for (k = 0; k < 3; k++) if (k != lo) {
          S[k][0] = S[lo][0] + 0.5 * (S[k][0] - S[lo][0]);
          S[k][1] = S[lo][1] + 0.5 * (S[k][1] - S[lo][1]);
          F[k] = gam_nll(h, mu, exp(S[k][0]), exp(S[k][1]));
        }
      }
    }
  }
  lo = 0;
  for (k = 1; k < 3; k++) if (F[k] < F[lo]) lo = k;
  *ret_mu = mu; *ret_lambda = exp(S[lo][0]); *ret_tau = exp(S[lo][1]);
  return eslOK;
}

/* binned exponential: geometric in the bin index, ML rate log(1+n/sum k)/w */
static int
fit_exp(const ESL_HISTOGRAM *h, double *ret_mu, double *ret_lambda)
{
  double n = 0.0, sk = 0.0;
  int b;
  for (b = h->cmin; b <= h->imax; b++) { n += (double)h->obs[b]; sk += (double)(b - h->cmin) * (double)h->obs[b]; }
  if (n <= 0) return eslFAIL;
  *ret_mu = h->phi;
  *ret_lambda = (sk > 0.0) ? log(1.0 + n / sk) / h->w : INFINITY;
  return eslOK;
}

/* cov_histogram_SetSurvFitTail, src/covariation.c:1676-1699 */
int
cov_histogram_SetSurvFitTail(ESL_HISTOGRAM *h, double **ret_survfit, double pmass,
                             double (*surv)(double x, void *params), void *params)
{
  double *sf = (double *)calloc((size_t)2 * h->nb, sizeof(double));
  int b;
  if (!sf) return eslEMEM;
  for (b = h->cmin; b < 2 * h->nb; b++) sf[b] = pmass * (*surv)(covh_Bin2UBound(h, b), params);
  *ret_survfit = sf;
  return eslOK;
}

/* cov_NullFitExponential, src/covariation.c:1914-1941 */
int
cov_NullFitExponential(ESL_HISTOGRAM *h, double **ret_survfit, double pmass, double *ret_newmass,
                       double *ret_mu, double *ret_lambda, int verbose, char *errbuf)
{
  double ep[2], newmass;
  (void)verbose;
  newmass = covh_SetTailByMass(h, pmass);
  if (fit_exp(h, &ep[0], &ep[1]) != eslOK) {
    if (errbuf) snprintf(errbuf, 256, "could not do exponential fit");
    return eslFAIL;
  }
  if (!isinf(ep[1])) cov_histogram_SetSurvFitTail(h, ret_survfit, newmass, covh_exp_surv, ep);
  *ret_mu = ep[0]; *ret_lambda = ep[1]; *ret_newmass = newmass;
  return eslOK;
}

/* cov_NullFitGamma, src/covariation.c:1943-1973 */
int
cov_NullFitGamma(ESL_HISTOGRAM *h, double **ret_survfit, double pmass, double *ret_newmass,
                 double *ret_mu, double *ret_lambda, double *ret_k, int verbose, char *errbuf)
{
  double ep[3], newmass;
  (void)verbose;
  newmass = covh_SetTailByMass(h, pmass);
  if (fit_gamma(h, &ep[0], &ep[1], &ep[2]) != eslOK) {
    if (errbuf) snprintf(errbuf, 256, "could not do a Gamma fit");
    return eslFAIL;
  }
  if (!isinf(ep[1])) cov_histogram_SetSurvFitTail(h, ret_survfit, newmass, covh_gamma_surv, ep);
  *ret_mu = ep[0]; *ret_lambda = ep[1]; *ret_k = ep[2]; *ret_newmass = newmass;
  return eslOK;
}

/* cov2evalue, src/covariation.c:2369-2400; an impossible bin returns +inf
 * where the reference exits */
double
covh_cov2evalue(double cov, double Nc, const ESL_HISTOGRAM *h, const double *survfit)
{
  int icov, i;
  uint64_t c = 0;
  if (covh_Score2Bin(h, cov, &icov) != eslOK) return INFINITY;
  if (survfit && icov >= 2 * h->nb - 1) return survfit[2 * h->nb - 1] * Nc;
  if (survfit && cov >= h->phi)         return survfit[icov + 1] * Nc;
  if (cov >= h->xmax) return Nc / (double)h->Nc;
  if (icov <= h->imax) {
    if (icov < h->imin) icov = h->imin;
    if (icov >= h->imax - 1) return Nc / (double)h->Nc;
    for (i = h->imax; i >= icov; i--) c += h->obs[i];
    return (double)c * Nc / (double)h->Nc;
  }
  return INFINITY;
}

/* evalue2cov, src/covariation.c:2403-2435 */
double
covh_evalue2cov(double eval_thresh, double Nc, const ESL_HISTOGRAM *h, const double *survfit)
{
  double cov = -INFINITY, eval;
  uint64_t c = 0;
  int b = h->cmin - 1, i;
  if (h->No >= 10 && survfit) {
    for (b = 2 * h->nb - 1; b >= h->cmin; b--) {
      eval = survfit[b] * Nc;
      if (eval >= eval_thresh) break;
    }
    cov = covh_Bin2LBound(h, b);
  }
  if (b == h->cmin - 1) {
    for (i = h->imax; i >= h->imin; i--) {
      c += h->obs[i];
      eval = (double)c * Nc / (double)h->Nc;
      if (eval >= eval_thresh) break;
    }
    cov = covh_Bin2UBound(h, i);
  }
  return cov;
}

/* cov_ranklist_Bin2Bin, src/covariation.c:2334-2362 */
int
cov_ranklist_Bin2Bin(int b, ESL_HISTOGRAM *h, ESL_HISTOGRAM *new_, int *ret_newb)
{
  double x = covh_Bin2LBound(h, b);
  if (!isfinite(x)) { *ret_newb = -1; return eslERANGE; }
  x = round((x - new_->bmin) / new_->w);
  if (x < -2147483647.0 || x > 2147483647.0) { *ret_newb = -1; return eslERANGE; }
  if ((int)x > new_->nb) { *ret_newb = -1; return eslERANGE; }
  *ret_newb = (int)x;
  return eslOK;
}

/* cov_CreateRankList, src/covariation.c:640-665 */
RANKLIST *
cov_CreateRankList(double bmax, double bmin, double w)
{
  RANKLIST *r = (RANKLIST *)calloc(1, sizeof(RANKLIST));
  if (!r) return NULL;
  r->ha = covh_Create(bmin, bmax, w);
  r->ht = covh_Create(bmin, bmax, w);
  r->hb = covh_Create(bmin, bmax, w);
  if (!r->ha || !r->ht || !r->hb) { cov_FreeRankList(r); return NULL; }
  r->survfit = NULL;
  return r;
}

void
cov_FreeRankList(RANKLIST *r)
{
  if (!r) return;
  covh_Destroy(r->ha); covh_Destroy(r->ht); covh_Destroy(r->hb);
  free(r->survfit);
  free(r);
}

void
cov_FreeHitList(HITLIST *h)
{
  if (!h) return;
  free(h->srthit);
  free(h->hit);
  free(h);
}

static void
copy_meta(ESL_HISTOGRAM *d, const ESL_HISTOGRAM *s)
{
  d->n = s->n; d->xmin = s->xmin; d->xmax = s->xmax; d->imin = s->imin; d->imax = s->imax;
  d->Nc = s->Nc; d->No = s->No;
}

/* cov_GrowRankList, src/covariation.c:682-736 */
int
cov_GrowRankList(RANKLIST **oranklist, double bmax, double bmin)
{
  RANKLIST *r = *oranklist, *nw;
  double new_bmin = r->ha->bmin;
  int b, nb;
  if (bmin < r->ha->bmin) new_bmin -= fabs(bmin) * 2. * r->ha->w;
  nw = cov_CreateRankList((bmax > r->ha->bmax) ? bmax : r->ha->bmax, new_bmin, r->ha->w);
  if (!nw) return eslEMEM;
  copy_meta(nw->ha, r->ha); copy_meta(nw->ht, r->ht); copy_meta(nw->hb, r->hb);
  for (b = r->ha->imin; b <= r->ha->imax; b++) {
    cov_ranklist_Bin2Bin(b, r->ha, nw->ha, &nb);
    if (nb >= 0 && nb < nw->ha->nb) nw->ha->obs[nb] = r->ha->obs[b];
  }
  cov_FreeRankList(r);
  *oranklist = nw;
  return eslOK;
}

/* cov_WriteNullHistogram, src/covariation.c:1844-1867: "score count" lines */
int
cov_WriteNullHistogram(char *nullhisfile, RANKLIST *ranklist, char *errbuf, int verbose)
{
  FILE *fp;
  int i;
  (void)verbose;
  if (ranklist == NULL) return eslOK;
  if ((fp = fopen(nullhisfile, "w")) == NULL) {
    if (errbuf) snprintf(errbuf, 256, "could not open nullhisfile %s", nullhisfile);
    return eslFAIL;
  }
  for (i = 0; i < ranklist->ha->nb; i++)
    fprintf(fp, "%f %llu\n", ranklist->ha->bmin + i * ranklist->ha->w, (unsigned long long)ranklist->ha->obs[i]);
  fclose(fp);
  return eslOK;
}

/* cov_ReadNullHistogram, src/covariation.c:1717-1842 */
int
cov_ReadNullHistogram(char *nullhisfile, RANKLIST **ret_ranklist, char *errbuf, int verbose)
{
  FILE     *fp;
  RANKLIST *r;
  char      line[1024];
  double    w = INFINITY, sc = -INFINITY, sc_prv, max_sc = -INFINITY, min_sc = INFINITY, bmin, bmax;
  double    tol = 1e-2;
  int       nread = 0;
  (void)verbose;
  if ((fp = fopen(nullhisfile, "r")) == NULL) {
    if (errbuf) snprintf(errbuf, 256, "file open failed");
    return eslFAIL;
  }
  while (fgets(line, sizeof(line), fp)) {
    double s; unsigned long long c;
    if (line[0] == '#') continue;
    if (sscanf(line, "%lf %llu", &s, &c) < 1) continue;
    sc_prv = sc; sc = s;
    if (fabs(sc - sc_prv) < w) w = fabs(sc - sc_prv);
    if (sc > max_sc) max_sc = sc;
    if (sc < min_sc) min_sc = sc;
    nread++;
  }
  if (nread < 2 || !(w > 0.0) || !isfinite(w)) {
    fclose(fp);
    if (errbuf) snprintf(errbuf, 256, "null histogram file %s: need at least two distinct scores", nullhisfile);
    return eslFAIL;
  }
  bmax = max_sc; bmin = min_sc;
  while (fabs(bmax - bmin) < tol) bmax += w;
  r = cov_CreateRankList(bmax, bmin, w);
  if (!r) { fclose(fp); return eslEMEM; }
  rewind(fp);
  while (fgets(line, sizeof(line), fp)) {
    double s; unsigned long long c; int b;
    ESL_HISTOGRAM *h = r->ha;
    if (line[0] == '#') continue;
    if (sscanf(line, "%lf %llu", &s, &c) != 2) continue;
    if (covh_Score2Bin(h, s, &b) != eslOK) { fclose(fp); cov_FreeRankList(r); return eslERANGE; }
    if (b < 0) {
      int nnew = -b * 2, i;
      uint64_t *o = (uint64_t *)calloc((size_t)h->nb + nnew, sizeof(uint64_t));
      if (!o) { fclose(fp); cov_FreeRankList(r); return eslEMEM; }
      memcpy(o + nnew, h->obs, sizeof(uint64_t) * h->nb);
      free(h->obs); h->obs = o;
      h->nb += nnew; b += nnew; h->bmin -= nnew * h->w; h->imin += nnew; h->cmin += nnew;
      if (h->imax > -1) h->imax += nnew;
      (void)i;
    } else if (b >= h->nb) {
      int nnew = (b - h->nb + 1) * 2, i;
      uint64_t *o = (uint64_t *)realloc(h->obs, sizeof(uint64_t) * ((size_t)h->nb + nnew));
      if (!o) { fclose(fp); cov_FreeRankList(r); return eslEMEM; }
      h->obs = o;
      for (i = h->nb; i < h->nb + nnew; i++) h->obs[i] = 0;
      if (h->imin == h->nb) { h->imin += nnew; h->cmin += nnew; }
      h->bmax += nnew * h->w; h->nb += nnew;
    }
    if (b < h->imin) { h->imin = b; h->cmin = b; }
    if (b > h->imax) h->imax = b;
    if (s < h->xmin) h->xmin = s;
    if (s > h->xmax) h->xmax = s;
    h->obs[b] = c;
    h->n += c; h->Nc += c; h->No += c;
  }
  fclose(fp);
  *ret_ranklist = r;
  return eslOK;
}

/* cov_Add2SubsHistogram, src/covariation.c:667-679: nsubs + 1 of every WWc
 * hit */
int
cov_Add2SubsHistogram(ESL_HISTOGRAM *hsubs, HITLIST *hitlist, int verbose)
{
  int h;
  (void)verbose;
  for (h = 0; h < hitlist->nhit; h++)
    if (hitlist->hit[h].bptype == WWc) covh_Add(hsubs, (double)(hitlist->hit[h].nsubs + 1));
  return eslOK;
}

/* cov_DumpRankList, src/covariation.c:738-754 (stdout, as the reference) */
int
cov_DumpRankList(FILE *fp, RANKLIST *ranklist)
{
  int b;
  (void)fp;
  if (ranklist == NULL) return eslOK;
  printf("imin %d imax %d covmin %f covmax %f\n", ranklist->ha->imin, ranklist->ha->imax, ranklist->ha->xmin,
         ranklist->ha->xmax);
  for (b = ranklist->ha->imax; b >= ranklist->ha->imin; b--) {
    double cov = covh_Bin2LBound(ranklist->ha, b);
    printf("cov %f eval %g\n", cov, covh_cov2evalue(cov, (double)ranklist->ha->Nc, ranklist->ha, NULL));
  }
  return eslOK;
}

/* cov_DumpHistogram, src/covariation.c:756-776 (stdout; the histograms here
 * carry no expected counts) */
int
cov_DumpHistogram(FILE *fp, ESL_HISTOGRAM *h)
{
  double nobs = 0.0, cum = 0.0;
  int b;
  (void)fp;
  for (b = h->imax; b >= h->imin; b--) nobs += (double)h->obs[b];
  printf("imin %d imax %d covmin %f covmax %f nobs %f\n", h->imin, h->imax, h->xmin, h->xmax, nobs);
  for (b = h->imax; b >= h->imin; b--) {
    cum += (double)h->obs[b];
    printf("b %d val %f obs %f cum_obs %f\n", b, covh_Bin2LBound(h, b), (double)h->obs[b], cum);
  }
  return eslOK;
}

/* cov_FisherExactTest, src/covariation.c:1584-1633: the one-sided sum of
 * hypergeometric probabilities from cNBP covarying pairs outside BP base
 * pairs up, log-factorials from lgamma (the reference uses Easel's) */
int
cov_FisherExactTest(double *ret_pval, int cBP, int cNBP, int BP, int alen)
{
  const int NBP = alen * (alen - 1) / 2, total = BP + NBP, cov = cBP + cNBP, non = total - cov;
  const double fixed = lgamma(BP + 1.0) + lgamma(NBP + 1.0) + lgamma(cov + 1.0) + lgamma(non + 1.0) - lgamma(total + 1.0);
  double pval = 0.0;
  int cnbp;
  for (cnbp = cNBP; cnbp <= NBP; cnbp++) {
    const int cbp = cov - cnbp, ncbp = BP - cbp, ncnbp = non - ncbp;
    if (cbp < 0) break;
    pval += exp(fixed - lgamma(cbp + 1.0) - lgamma(ncbp + 1.0) - lgamma(cnbp + 1.0) - lgamma(ncnbp + 1.0));
  }
  if (pval > 1.0 && pval < 1.0 + 1e-3) pval = 1.0;
  *ret_pval = pval;
  return eslOK;
}

/* cov_histogram_PlotSurvival, src/covariation.c:1636-1676: the observed
 * survival (largest value first, then every non-empty bin's lower bound
 * with the fraction at or above it), "&", and the fitted survival when
 * given, "&" */
int
cov_histogram_PlotSurvival(FILE *fp, ESL_HISTOGRAM *h, double *survfit)
{
  uint64_t c = 0;
  int i;
  if (h->imax >= 0 && h->obs[h->imax] > 1)
    if (fprintf(fp, "%f\t%g\n", h->xmax, 1.0 / (double)h->Nc) < 0) return eslFAIL;
  for (i = h->imax; i >= h->imin; i--)
    if (h->obs[i] > 0) {
      c += h->obs[i];
      if (fprintf(fp, "%f\t%g\n", covh_Bin2LBound(h, i), (double)c / (double)h->Nc) < 0) return eslFAIL;
    }
  if (fprintf(fp, "&\n") < 0) return eslFAIL;
  if (survfit) {
    for (i = 2 * h->nb - 1; i >= 0; i--)
      if (survfit[i] > 0.)
        if (fprintf(fp, "%f\t%g\n", covh_Bin2LBound(h, i), survfit[i]) < 0) return eslFAIL;
    if (fprintf(fp, "&\n") < 0) return eslFAIL;
  }
  return eslOK;
}
