/* rscape_oracle.h -- CPU FP64 oracle for the R-scape covariation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C and double
 * precision, the reference algorithms of R-scape 2.6.11's covariation path
 * (src/correlators.c, src/covariation.c, src/R-scape.c null loop,
 * src/msatree.c Fitch, src/msamanip.c substitution shuffle).  It is the
 * checker for the GPU library: only the tests, the smoke check and the
 * CPU-baseline leg of the benchmark may load it.  Nothing in the shipped
 * GPU library links, calls or falls back to it.
 *
 * Parity status: counting, marginals, GTp and APC are pinned by the golden
 * GTp scores published for tutorial/updated_Arisong.sto
 * (documentation/tutorial.tex:186-212).  The
 * Easel pieces (sequence weights, histogram binning, binned tail fits, RNG)
 * are absent from the reference tree and are restated from their published
 * mathematics; E-values are therefore pinned only against this oracle's own
 * restatement, not against a stock R-scape build.
 *
 * Data conventions (shared with the GPU library):
 *   ax    uint8 row-major [N][L], Easel RNA digital codes: 0..3 = ACGU,
 *         4 = gap, 5..14 degenerate, 15 = N, 16 = '*', 17 = '~'.
 *   wgt   double [N] sequence weights.
 *   trees follow Easel's ESL_TREE convention: N leaves, N-1 internal nodes,
 *         node 0 is the root, parent[v] < v, left/right > 0 = internal node,
 *         <= 0 = leaf -value.
 */
#ifndef RSCAPE_ORACLE_H
#define RSCAPE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* covariation types: same numbering as COVTYPE (src/correlators.h:45-79) */
enum { ORC_CHI = 0, ORC_GT = 3, ORC_MI = 6, ORC_MIr = 9, ORC_MIg = 12, ORC_OMES = 15,
       ORC_RAF = 18, ORC_RAFS = 21, ORC_CCF = 24 };
/* classes: COVCLASS (src/correlators.h:38-43) */
enum { ORC_C16 = 0, ORC_C2 = 1, ORC_CWC = 2, ORC_CSELECT = 3 };
/* corrections: ACTYPE (src/correlators.h:81-84) */
enum { ORC_APC = 0, ORC_ASC = 1 };

typedef struct {
  int           N;           /* leaves */
  const int    *parent;      /* [N-1] */
  const int    *left;        /* [N-1] */
  const int    *right;       /* [N-1] */
  const double *ld;          /* [N-1] */
  const double *rd;          /* [N-1] */
} orc_tree_t;

typedef struct {
  double    bmin, bmax, w;
  int       nb;
  uint64_t *obs;
  uint64_t  n, Nc, No;
  double    xmin, xmax;
  int       imin, imax, cmin;
  double    phi;
} orc_hist_t;

/* parameters of one R-scape run (defaults of src/R-scape.c:254-433, 883-892) */
typedef struct {
  int    covtype;        /* e.g. ORC_GT+1 = GTp */
  int    covclass;       /* ORC_CSELECT by default */
  int    nseqthresh;     /* 8 */
  int    alenthresh;     /* 50 */
  int    nshuffle;       /* <0: R-scape's rule (src/R-scape.c:2449-2456) */
  double thresh;         /* E-value threshold, 0.05 */
  double bmin;           /* -10 */
  double w0;             /* 0.05 */
  int    hpts;           /* 400 */
  double pmass;          /* 0.0005 */
  double fracfit;        /* 1.0 */
  int    doexpfit;       /* 0 = gamma */
  double tol;            /* 1e-6 */
  uint64_t seed;         /* 42 */
  double allow[16];      /* allowed pairs, row-major 4x4 */
  /* the two-set test (R-scape -s, src/R-scape.c:1139-1160) and
   * --structured (:1911-1918) */
  int            samplesize;  /* ORC_SAMPLE_ALL (one-set test) by default */
  int            ncnt;        /* contacts of the given structure */
  const int64_t *cnt_i;       /* [ncnt] 1-based alignment positions */
  const int64_t *cnt_j;
  const int     *cnt_type;    /* [ncnt] BPTYPE */
  int            mind;        /* with msa2pdb: pairs closer than mind in the PDB are not ranked */
  const int     *msa2pdb;     /* [L] or NULL */
  double         expBP;       /* -1 by default */
} orc_params_t;

enum { ORC_SAMPLE_CONTACTS = 0, ORC_SAMPLE_BP = 1, ORC_SAMPLE_WC = 2, ORC_SAMPLE_ALL = 3 };
enum { ORC_WWc = 0, ORC_STACKED = 32, ORC_CONTACT = 33, ORC_BPNONE = 34 };

typedef struct {
  int      nshuffle;
  double   w;             /* histogram width from the first null */
  double   null_minCOV, null_maxCOV;
  double   minCOV, maxCOV; /* of the real alignment after correction */
  double   pmass_used, newmass, mu, lambda, tau;
  int      fit_ok;
  double   sc_thresh;     /* evalue2cov threshold (of base pairs in the two-set test: sc_bp) */
  uint64_t Nt;            /* number of tests (of the pairs outside the structure in the two-set test) */
  int      nhit;
  /* null histogram metadata */
  double   h_bmin, h_w;
  int      h_nb, h_imin, h_imax, h_cmin;
  uint64_t h_n, h_Nc, h_No;
  double   h_xmin, h_xmax, h_phi;
  double   sc_nbp;        /* threshold of the pairs outside the structure */
  uint64_t Nb;            /* number of tests of the base pairs (0 in the one-set test) */
} orc_result_t;

/* ---- RNG: Philox4x32-10 (Salmon et al., SC'11) ---- */
void orc_philox4x32(const uint32_t key[2], const uint32_t ctr[4], uint32_t out[4]);

/* ---- weights and MSA preparation ---- */
int  orc_weights_pb (const uint8_t *ax, int N, int L, double *wgt);
int  orc_weights_gsc(const uint8_t *ax, int N, int L, double *wgt);
int  orc_gapfilter  (const uint8_t *ax, const double *wgt, int N, int L, double gapthresh, int *useme);
void orc_degen2n    (uint8_t *ax, int64_t n);

/* ---- probabilities (src/correlators.c:1300-1375, 1423-1545, 1695-1817) ---- */
int  orc_probs(const uint8_t *ax, const double *wgt, int N, int L, double tol,
               double *pp, double *nseff, double *ngap, double *pm, double *ps);

/* ---- statistics (src/correlators.c:49-1157) ---- */
int  orc_stat(int stat, int covclass, int N, int L, int nseqthresh, int alenthresh,
              const double *pp, const double *pm, const double *nseff, const double *ngap,
              const double *allow, double *COV, double *minmax);
int  orc_raf (const uint8_t *ax, int N, int L, const double *allow, double *COV, double *minmax);
int  orc_rafs(const uint8_t *ax, int N, int L, const double *allow, double *COV, double *minmax);
int  orc_ccf (int L, const double *pm, const double *nseff, double *COV, double *minmax);
int  orc_cov_corrected(int actype, int L, double *COV, double *minmax);
int  orc_cov_calculate(int covtype, int covclass, const uint8_t *ax, const double *wgt, int N, int L,
                       int nseqthresh, int alenthresh, const double *allow, double tol,
                       double *COV, double *minmax);

/* ---- histograms (Easel histogram semantics restated) ---- */
orc_hist_t *orc_hist_create(double bmin, double bmax, double w);
void        orc_hist_free(orc_hist_t *h);
int         orc_hist_score2bin(const orc_hist_t *h, double x);
double      orc_hist_lbound(const orc_hist_t *h, int b);
double      orc_hist_ubound(const orc_hist_t *h, int b);
int         orc_hist_add(orc_hist_t *h, double x);

/* ---- null alignments (src/msatree.c:173-227,1700-1931; src/msamanip.c:1164-1233,1449-1780) ---- */
uint32_t orc_feistel_perm(uint32_t t, uint32_t L, const uint32_t rk[6]);
int  orc_fitch(const uint8_t *ax, int N, int L, const orc_tree_t *T, uint64_t seed, uint32_t null_id,
               uint8_t *allmsa);
int  orc_null_msa(const uint8_t *ax, int N, int L, const orc_tree_t *T, uint64_t seed, uint32_t null_id,
                  uint8_t *out_ax);

/* ---- P(t) alignment simulator (src/cov_simulate.c:288-451,586-798; src/ratematrix.c:185-233) ---- */
/* P = exp(t Q) for an n x n rate matrix: scaling and squaring of a Taylor series */
int  orc_sim_expm(const double *Q, int n, double t, double *P);
/* ratematrix_ConditionalsFromRate: P(t) with the reference's time rules, small
 * negative entries zeroed (others fail), rows renormalised */
int  orc_sim_conditionals(const double *Q, int n, double rt, double *P);
/* inverse-CDF thresholds of the n rows of P: C[i][k] = floor(cdf 2^64) of the
 * running sum, the last of each row 2^64 - 1 */
void orc_sim_cdf(const double *P, int n, int nrows, uint64_t *C);
/* one alignment [N][L]: root (or a draw from the root CDFs R4/R16 when root
 * is NULL) evolved down T with the per-branch thresholds C4 [2(N-1)][4][4]
 * and C16 [2(N-1)][16][16] (branch 2v + side), ct[c] = partner or -1, then
 * gap runs; rep selects the replicate's random streams */
int  orc_simulate(const orc_tree_t *T, int N, int L, const int *ct, const uint64_t *C4, const uint64_t *C16,
                  const uint64_t *R4, const uint64_t *R16, const uint8_t *root, double gap_rate,
                  double gap_mean, uint64_t seed, uint32_t rep, uint8_t *out);

/* ---- substitutions and power (src/msatree.c:1423-1554; src/power.c:65-218) ---- */
int    orc_substitutions(const uint8_t *ax, int N, int L, const orc_tree_t *T, uint64_t seed, uint32_t null_id,
                         int includegaps, int *nsubs, int *ndouble, int *njoin);
double orc_power_step(double n, int ns, const double *subs, const double *prob);

/* ---- the whole per-alignment path (src/R-scape.c:1281-1371, 1564-1724, 2335-2724) ---- */
void orc_params_default(orc_params_t *p);
int  orc_rscape(const orc_params_t *p, const uint8_t *ax, const double *wgt, int N, int L,
                const orc_tree_t *T,
                double *COV, double *Eval,                 /* [L*L] or NULL */
                uint64_t *null_obs, int null_obs_cap,      /* cumulative null histogram */
                int *hit_i, int *hit_j, double *hit_sc, double *hit_E, double *hit_p, int hit_cap,
                orc_result_t *res);
/* orc_rscape for nt statistics sharing the nulls; per-statistic outputs in nt
 * consecutive blocks (COV/Eval L*L, null_obs null_obs_cap, hits hit_cap) */
int  orc_rscape_multi(const orc_params_t *p, int nt, const int *covtypes, const uint8_t *ax, const double *wgt,
                      int N, int L, const orc_tree_t *T, double *COV_out, double *Eval_out, uint64_t *null_obs,
                      int null_obs_cap, int *hit_i, int *hit_j, double *hit_sc, double *hit_E, double *hit_p,
                      int hit_cap, orc_result_t *res);

/* ---- reference-faithful timing mode (per-pair column gathers, FP64) ---- */
double orc_faithful_rows(const uint8_t *ax, const double *wgt, int N, int L, int i0, int i1,
                         int nthreads, double *checksum);
double orc_faithful_raf(const uint8_t *ax, int N, int L, int npairs, int nthreads, double *checksum);

/* RAF (the reference's O(N^2) loop) of listed pairs only, on the host threads */
void   orc_raf_pairs(const uint8_t *ax, int N, int L, const double *allow, int npairs, const int *pi, const int *pj,
                     double *out);

/* ---- learned null (the library's own definitions; no reference counterpart) ----
 * feat[64] of ax [N][L] with weights w: the alignment features 0-46 of the
 * library's covgpu_features, computed here in FP64 in sequence order
 * (47-63, the null-score summary, are 0). */
void   orc_features(const uint8_t *ax, int N, int L, const double *w, double tree_len, double *feat);
/* the 64-256-256-256-3 SiLU network with FP32 master parameters params
 * (weights rounded to BF16 by round-to-nearest-even, biases as given) and
 * standardisation nrm = xmean[64] xstd[64] ymean[3] ystd[3], in FP64:
 * Y[n][3] de-standardised outputs; orc_mlp_grad returns the mean squared
 * error on standardised targets and its gradient grad[148995] */
void   orc_mlp_forward(const float *params, const float *nrm, const float *X, int n, double *Y);
double orc_mlp_grad(const float *params, const float *nrm, const float *X, const float *T, int n, double *grad);

/* corr_CalculateRAF from unit counts (exact; the deep-alignment form of orc_raf) */
int    orc_raf_counts(const uint8_t *ax, int N, int L, const double *allow, double *COV, double *minmax);

/* helix aggregation (src/aggregate.c:146-322, 375-488) */
double orc_agg_fisher(int n, const double *p);
double orc_agg_weighted(int n, const double *p, const double *w);   /* Lancaster and weighted Fisher */
double orc_agg_sidak(int n, const double *p);
void   orc_agg_weights_lancaster(int n, const double *nsubs, double *w);
void   orc_agg_weights_wfisher(int n, const double *power, double *w);

#ifdef __cplusplus
}
#endif

#endif
