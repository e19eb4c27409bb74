/* covgpu.h -- batched C-ABI of the GB300 covariation engine (libcovgpu.so).
 *
 * One context owns the device buffers for alignments of N sequences x L
 * columns (after R-scape's gap-column filter) and up to `maxslots` of them at
 * once: slot 0 is normally the input alignment, slots 1..nshuffle its null
 * alignments.  All arguments are plain pointers and sizes; host buffers are
 * ordinary (or pinned) host memory.  Every call returns 0 on success or a
 * nonzero status with a message in the context's error buffer
 * (covgpu_errmsg); a NULL context (or batch, or network) returns 11.
 *
 * This is the fast path behind the reference-named entry points of
 * rscape_cov.h: one call of covgpu_rscape() does what R-scape's
 * rscape_for_msa() does for the covariation part (src/R-scape.c:2335-2544):
 * null alignments (null_rscape, :1614-1724), histogram width
 * (calculate_width_histo, :1281-1371), scoring of every alignment
 * (cov_Calculate, src/covariation.c:63-306), the null histogram, the tail fit
 * and the E-values of the input alignment (cov_SignificantPairs_Ranking and
 * cov_CreateHitList, :325-530, :778-1006).
 */
#ifndef COVGPU_H
#define COVGPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct covgpu_ctx covgpu_ctx;

/* counting kernels */
enum { COVGPU_COUNT_SIMT = 0, COVGPU_COUNT_TENSOR = 1 };

typedef struct {
  int      covclass;     /* COVCLASS: 0 C16, 1 C2, 2 CWC, 3 CSELECT (default 3) */
  int      nseqthresh;   /* 8 */
  int      alenthresh;   /* 50 */
  int      nshuffle;     /* < 0: R-scape's rule (src/R-scape.c:2449-2456) */
  double   thresh;       /* E-value threshold (0.05) */
  double   bmin;         /* -10 */
  double   w0;           /* 0.05 */
  int      hpts;         /* 400 */
  double   pmass;        /* 0.0005 */
  double   fracfit;      /* 1.0 */
  int      doexpfit;     /* 0 = gamma tail, 1 = exponential tail */
  double   tol;          /* 1e-6 */
  uint64_t seed;         /* 42 */
  double   allow[16];    /* allowed pairs (AU UA CG GC GU UG) */
  int      counter;      /* COVGPU_COUNT_SIMT or COVGPU_COUNT_TENSOR */
  /* the two-set test (R-scape -s) and --structured, covgpu_rscape only:
   * the given structure's contacts, 1-based alignment positions
   * cnt_i[h] < cnt_j[h] with their BPTYPE (WWc = 0 ... 31, STACKED 32,
   * CONTACT 33, BPNONE 34), as R-scape's CLIST holds them */
  int             samplesize;  /* 3 (default): one-set test; 0 contacts, 1 base pairs, 2 WC pairs */
  int             ncnt;        /* 0 (default): no structure */
  const int64_t  *cnt_i, *cnt_j;
  const int      *cnt_type;
  double          expBP;       /* --structured: expected base pairs; <= 0 (default -1) off */
} covgpu_params;

typedef struct {
  int      covtype;       /* COVTYPE code, e.g. 4 = GTp */
  int      status;        /* 0 ok; 1 scores constant (w == 0); 2 one sequence */
  int      nshuffle;
  double   w;             /* histogram width fixed by the first null */
  double   minCOV, maxCOV;          /* input alignment, after correction */
  double   null_minCOV, null_maxCOV; /* first null */
  double   pmass, newmass, mu, lambda, tau;
  double   sc_thresh;     /* score at the E-value threshold (of base pairs in the two-set test: sc_bp) */
  uint64_t Nt;            /* number of tests (of the pairs outside the structure in the two-set test) */
  int      nhit;          /* pairs with E < thresh (may exceed hitcap) */
  /* cumulative null histogram */
  double   h_bmin, h_w, h_xmin, h_xmax, h_phi;
  int      h_nb, h_imin, h_imax, h_cmin;
  uint64_t h_n, h_Nc, h_No;
  double   sc_nbp;        /* score at the E-value threshold of the pairs outside the structure */
  uint64_t Nb;            /* number of tests of the base pairs (0 in the one-set test) */
} covgpu_result;

typedef struct {
  int    i, j;            /* 0-based columns of the filtered alignment, i < j */
  double sc, E, pval;
} covgpu_hit;

void        covgpu_params_default(covgpu_params *p);
const char *covgpu_errmsg(const covgpu_ctx *ctx);

int  covgpu_create(covgpu_ctx **ret, int device, int N, int L, int maxslots, int maxnull);
void covgpu_destroy(covgpu_ctx *ctx);
/* switch the context to alignments of N x L, N and L at most those it was
 * created for, without allocating: for streams of families of different
 * sizes.  Alignment, weights and tree must be set again afterwards. */
int  covgpu_resize(covgpu_ctx *ctx, int N, int L);

/* inputs: codes are Easel RNA digital codes, row-major [N][L] */
int  covgpu_set_weights(covgpu_ctx *ctx, const double *wgt);
int  covgpu_set_alignment(covgpu_ctx *ctx, int slot, const uint8_t *ax);
int  covgpu_get_alignment(covgpu_ctx *ctx, int slot, uint8_t *ax);
/* Easel ESL_TREE convention: node 0 root, parent[v] < v, children > 0 are
 * internal nodes, <= 0 are leaves -value; arrays of N-1 entries */
int  covgpu_set_tree(covgpu_ctx *ctx, const int *parent, const int *left, const int *right);
/* null alignments null_id = first_null .. first_null+nnull-1 of the
 * alignment in slot 0, written to slots first_slot .. */
int  covgpu_make_nulls(covgpu_ctx *ctx, uint64_t seed, int first_null, int nnull, int first_slot);

/* P(t) alignment simulator on the device (replaces cov_GenerateAlignment's
 * ungapped evolution, src/cov_simulate.c:61-159,288-324,388-451,586-798,
 * with ratematrix_ConditionalsFromRate, src/ratematrix.c:185-233): nrep
 * alignments evolved down the context's tree (covgpu_set_tree) with branch
 * lengths ld/rd [N-1], written to slots first_slot .. first_slot+nrep-1.
 * Unpaired columns follow the 4x4 rate matrix Q4 (row-major, ACGU), base
 * pairs the 16x16 pair rate matrix Q16 (state 4x+y); ct[L] = partner column
 * or -1.  The root is root[L] (canonical residues) or, when NULL, drawn from
 * the backgrounds pi4 / pi16.  Then each leaf row gets gap runs: a gapped
 * column continues its run with probability 1 - 1/gap_mean, any other
 * column opens one with probability gap_rate/gap_mean (gap_rate 0: none).
 * Replicate r uses the random streams of replicate id rep0 + r.  Returns 0,
 * 11 (bad arguments), 41/42 (a branch time or P(t) the reference rejects). */
int  covgpu_simulate(covgpu_ctx *ctx, const double *ld, const double *rd, const double *Q4, const double *pi4,
                     const double *Q16, const double *pi16, const int *ct, const uint8_t *root, double gap_rate,
                     double gap_mean, uint64_t seed, uint32_t rep0, int first_slot, int nrep);
/* alignment preparation on the device, for the alignment in a slot:
 * position-based weights (Henikoff & Henikoff 1994; esl_msaweight_PB, which
 * R-scape uses for nseq > 1000, src/R-scape.c:1556) summing to N, written to
 * wgt[N] and, with set != 0, made the context's weights; and R-scape's gap
 * column filter (msamanip_RemoveGapColumns, src/msamanip.c:461-501):
 * useme[c] = 1 to keep column c (wgt NULL: unit weights) */
int  covgpu_weights_pb_dev(covgpu_ctx *ctx, int slot, int set, double *wgt);
/* Gerstein/Sonnhammer/Chothia tree weights (esl_msaweight_GSC, R-scape's
 * choice for nseq <= 1000, src/R-scape.c:1555) on the device: distances
 * 1 - identities/min(residues), UPGMA, each new branch shared among the
 * leaves below it in proportion to their weights; summing to N */
int  covgpu_weights_gsc_dev(covgpu_ctx *ctx, int slot, int set, double *wgt);
int  covgpu_gapfilter_dev(covgpu_ctx *ctx, int slot, const double *wgt, double gapthresh, int *useme);
/* substitutions on the branches of the context's tree (Tree_Substitutions,
 * src/msatree.c:1423-1554) for the alignment in slot, on its Fitch
 * reconstruction (random tie-breaks from seed): nsubs[L] per column; ndouble
 * and njoin [L][L] per pair i < j (upper triangle, the rest 0): branches
 * where both / at least one of the columns change; both ends canonical unless
 * includegaps.  Outputs may be NULL; the last result stays on the device for
 * covgpu_power. */
int  covgpu_substitutions(covgpu_ctx *ctx, int slot, uint64_t seed, int includegaps, int *nsubs, int *ndouble,
                          int *njoin);
/* power of every pair i < j, in row-major order of the upper triangle
 * (power_SPAIR_Create, src/power.c:65-218): the probability of the last of
 * the ns curve points whose substitution count the pair's exceeds, for the
 * single (nsubs_i + nsubs_j), join and double counts; a curve given as NULL
 * gives 0 (single) or -1 (join, double) */
int  covgpu_power(covgpu_ctx *ctx, int ns, const double *subs, const double *prob, const double *subs_join,
                  const double *prob_join, const double *subs_double, const double *prob_double, double *power,
                  double *power_join, double *power_double);
/* the pair classes of power_SPAIR_AddMI (src/power.c:201-218) from the
 * weighted counts of the last covgpu_score/covgpu_rscape of slot, without
 * the pair probabilities on the host: per pair i < j (row-major over the
 * upper triangle, L(L-1)/2 each) the Watson-Crick fraction pp(AU) + pp(UA) +
 * pp(CG) + pp(GC), the wobble fraction pp(GU) + pp(UG) and the rest, with
 * pp = (1e-10 + C)/sum as covgpu_get_probs gives it; any pointer may be NULL */
int  covgpu_pair_classes(covgpu_ctx *ctx, int slot, double *wcf, double *wobble, double *noncan);
/* the per-branch conditionals of the last covgpu_simulate: P4 [2(N-1)][4][4]
 * and P16 [2(N-1)][16][16], branch 2v (left child of v) and 2v+1 (right) */
int  covgpu_sim_tables(covgpu_ctx *ctx, double *P4, double *P16);

/* scores: covtypes are COVTYPE codes (CHI=0, CHIp=1, CHIa=2, GT=3, GTp=4,
 * ... CCFa=26), at most 4 per call; minmax[slot][type][2] on return */
int  covgpu_score(covgpu_ctx *ctx, int first_slot, int nslots, int ntypes, const int *covtypes, int covclass,
                  int nseqthresh, int alenthresh, const double *allow, int counter, double *minmax);
/* covgpu_score that reuses the weighted counts a previous score of the same
 * slots (same counter) left on the device, when no call since has changed
 * those alignments, the weights or the count buffer; otherwise it counts as
 * covgpu_score does.  (corr_Probs then corr_Calculate* on one alignment
 * count once.) */
int  covgpu_score_reuse(covgpu_ctx *ctx, int first_slot, int nslots, int ntypes, const int *covtypes, int covclass,
                        int nseqthresh, int alenthresh, const double *allow, int counter, double *minmax);
/* full L x L score matrix of one (slot, type index of the last covgpu_score),
 * diagonal -inf, both triangles (the layout of mi->COV) */
int  covgpu_get_cov(covgpu_ctx *ctx, int slot, int which, double *COV);
/* probabilities of one slot after covgpu_score: any pointer may be NULL.
 * nseff, ngap [L*L]; pm [L*4]; ps [L*5]; pp [L*L*16] */
int  covgpu_get_probs(covgpu_ctx *ctx, int slot, const double *wgt, double *pp, double *nseff, double *ngap,
                      double *pm, double *ps);

/* the whole per-alignment path for up to 4 covariation types sharing the
 * same null alignments.  results[ntypes]; hits[ntypes * hitcap].  ax == NULL
 * or wgt == NULL reuse the alignment in slot 0 / the weights already set;
 * the tree must have been set with covgpu_set_tree. */
int  covgpu_rscape(covgpu_ctx *ctx, const covgpu_params *p, const uint8_t *ax, const double *wgt,
                   int ntypes, const int *covtypes, covgpu_result *results, covgpu_hit *hits, int hitcap);

/* ---- the E-valued path over a batch of alignment families ----
 * A family is one input alignment with its tree; families differ in N, L and
 * null count.  covgpu_rscape_families does for every family what
 * covgpu_rscape does for one (the same nulls for the same seed, the same
 * statistics, histograms, tail fits and E-values), with every device pass
 * one grouped launch over the families: GSC or position-based weights
 * (R-scape's rule, src/R-scape.c:1545-1562, where wgt is NULL), the nulls
 * (one launch per tree depth over every family), the counts (one persistent
 * tensor-core launch over every family's tiles), the statistics and APC/ASC,
 * the null histograms, the tail fits (one block per fit), the survival
 * tables and the E-values; the host steps run once per phase for all
 * families.  Families are processed in chunks that fit the batch's device
 * budget (mem_gb; 0: a quarter of the free memory); the device passes of a
 * chunk run as a CUDA graph, replayed while the chunk's layout repeats. */
typedef struct covgpu_batch covgpu_batch;
typedef struct {
  int            N, L;
  const uint8_t *ax;       /* N x L codes, row-major */
  const double  *wgt;      /* N weights, or NULL: R-scape's rule on the device */
  const int     *parent;   /* the tree (covgpu_set_tree convention), N-1 entries each; */
  const int     *left;     /* parent may be NULL */
  const int     *right;
} covgpu_family;
int  covgpu_batch_create(covgpu_batch **ret, int device, double mem_gb);
void covgpu_batch_destroy(covgpu_batch *b);
const char *covgpu_batch_errmsg(const covgpu_batch *b);
/* results[nfam * ntypes] (family-major); hits[nfam * ntypes * hitcap];
 * returns 0 or the first error (its message names the family) */
int  covgpu_rscape_families(covgpu_batch *b, const covgpu_params *p, int nfam, const covgpu_family *fams,
                            int ntypes, const int *covtypes, covgpu_result *results, covgpu_hit *hits, int hitcap);
/* the count schedule: families of fewer than simt_below sequences are
 * counted on the SIMT kernel when the tensor counter is asked for (the counts
 * are the same), sb the raster super-block of the tensor count's tile order
 * (a square or a band, as in covgpu_autotune; defaults 64 and 10; 11 for a
 * bad value); covgpu_batch_autotune times the caller's families
 * under every (thr[i], sbs[j]) pair (host wall clock, best of two calls
 * after a warm-up; ms[i * nsb + j]) and keeps the fastest */
int  covgpu_batch_set_schedule(covgpu_batch *b, int simt_below, int sb);
int  covgpu_batch_autotune(covgpu_batch *b, const covgpu_params *p, int nfam, const covgpu_family *fams,
                           int ntypes, const int *covtypes, int nthr, const int *thr, int nsb, const int *sbs,
                           double *ms, int *best_thr, int *best_sb);
/* the last call: device milliseconds of [0] the passes from the nulls to the
 * corrected scores, [1] the histograms, fits and E-values (with their host
 * steps), [2] host wall clock of the whole call; kernel launches; chunks */
int  covgpu_batch_timing(const covgpu_batch *b, double *ms3, int *nlaunch, int *nchunks);

/* device timing of the last covgpu_rscape phases, milliseconds:
 * [0] nulls [1] counts [2] statistics+correction [3] histograms+fit+E-values
 * [4] total; also the number of kernel launches */
int  covgpu_last_timing(const covgpu_ctx *ctx, double *ms5, int *nlaunch);

/* ---- single-matrix steps behind the reference-named entry points ----
 * COV is a full L x L host matrix (both triangles); NULL uses the device's
 * latest score matrix of slot 0. */
/* validation of the pair probabilities of slot 0 (corr_ValidateProbs,
 * src/correlators.c:1499-1545) on the device: every pair's 16 probabilities
 * (prior 1e-10, from the counts of the last covgpu_score) in [0, 1 + tol] and
 * summing to 1 within tol.  Returns 0, or 20 when a pair fails. */
int  covgpu_validate_probs(covgpu_ctx *ctx, double tol);
/* APC (actype 0) or ASC (1) of COV into out (may alias COV or be NULL);
 * minmax[2] of the corrected off-diagonal scores */
int  covgpu_correct(covgpu_ctx *ctx, const double *COV, int actype, double *out, double *minmax);
/* counts of max(COV_ij, bmin + w), i < j, in nb bins of width w from bmin */
int  covgpu_hist_full(covgpu_ctx *ctx, const double *COV, double bmin, double w, int nb, uint64_t *obs);
/* E-values of every pair against a null histogram h (+ survfit, may be NULL),
 * times Nt tests; Eval full L x L (may be NULL); pairs with E < thresh */
int  covgpu_evalue_full(covgpu_ctx *ctx, const double *COV, const void *h, const double *survfit, double Nt,
                        double thresh, double *Eval, covgpu_hit *hits, int hitcap, int *nhit);
/* page-lock (pin) a host array the caller copies to and from the device,
 * and undo it before the array is freed; 0, or 90 when the driver refuses
 * (the copies then run unpinned) */
int  covgpu_host_pin(void *p, size_t bytes);
void covgpu_host_unpin(void *p);
/* covgpu_evalue_full with the two-set test and --structured
 * (cov_CreateHitList, src/covariation.c:828-870): pair n = i (2L - i - 1)/2
 * + j - i - 1 takes Nb tests when bit n of bpmask (may be NULL) is set; any
 * other pair takes expBP tests while fewer than expBP pairs before it in
 * scan order are hits (expBP <= 0: never), else Nt.  Hits come in scan
 * order. */
int  covgpu_evalue_sets(covgpu_ctx *ctx, const double *COV, const void *h, const double *survfit, double Nt,
                        double Nb, double expBP, const uint32_t *bpmask, double thresh, double *Eval,
                        covgpu_hit *hits, int hitcap, int *nhit);

/* APC (actype 0) or ASC (1) of a device-resident L x L score matrix (both
 * triangles; the diagonal is ignored) into the device buffer d_out (diagonal
 * set to -inf), with the min/max of the corrected scores in d_minmax[2],
 * enqueued on `stream` (a cudaStream_t; NULL = the legacy default stream).
 * d_out may be d_cov (in place); otherwise the two must not overlap.
 * No counterpart in the reference: this entry point allocates no device
 * memory, for callers that cannot call cudaMalloc (code running inside a
 * stream capture, pooled-memory hosts, real-time callers).  Its scratch is a
 * fixed device array sized for L <= COVGPU_NOALLOC_MAX_L; larger L returns
 * 11.  The first call on a device (and the first after the device's context
 * was recreated, e.g. by a device reset) looks up that array's device
 * address, so make it before any stream capture.  All calls share the
 * array: calls that overlap on the GPU race and must be serialised by the
 * caller.  Returns 0, 11 (bad arguments) or 90 (CUDA error).  The work is
 * asynchronous, so a NaN among the corrected scores (an error in the
 * reference, "bad covariation") is reported in the result: d_minmax is
 * then {NaN, NaN}. */
#define COVGPU_NOALLOC_MAX_L 16384
int  covgpu_correct_noalloc(const double *d_cov, double *d_out, int L, int actype, double *d_minmax, void *stream);

/* schedule autotuner of the tensor count kernel: times the weighted count of
 * slots first_slot .. first_slot+nslots-1 (weights set) for each raster
 * super-block in cand[ncand] and keeps the fastest for the context's later
 * calls.  The resident CTAs sweep super-blocks of tiles so they share operand
 * rows in L2: a value v < 1000 is a square of v x v tiles, v = 1000 a + b a
 * band a tile rows high and b columns wide (NULL: 4, 6, 8, 10, 12, 16, 24,
 * 32004, 48004, 48008, 96004).  Returns the median milliseconds of each in ms
 * (may be NULL) and the choice in *best.  The count buffer is overwritten. */
int  covgpu_autotune(covgpu_ctx *ctx, int first_slot, int nslots, int ncand, const int *cand, float *ms, int *best);
/* host code (no device): the tensor count's task orders for a schedule value
 * (as in covgpu_autotune) on nT column tiles of 32 columns.  order[nT(nT+1)/2]
 * receives the weighted kernel's tiles (indices into the row-major list of
 * tiles I <= J); jpairs[4 * jcap] (may be NULL) the unit-weight kernel's
 * tasks {I, J0, tile (I, J0), tile (I, J0 + 1)} (-1 for a tile outside
 * I <= J < nT) and *njpairs their number.  Returns 0, or 11 (bad schedule,
 * nT < 1, jcap too small). */
int  covgpu_tile_order(int nT, int schedule, int *order, int *jpairs, int jcap, int *njpairs);

/* writes a 256 MB device buffer (larger than L2) on the context's stream */
int  covgpu_flush_l2(covgpu_ctx *ctx);

/* ---- learned null (no counterpart in the reference) ----
 * R-scape gets the null score tail of every alignment from simulated null
 * alignments (null_rscape, src/R-scape.c:1614-1724, and the gamma fit of
 * cov_NullFitGamma, src/covariation.c:1943-1973).  The learned null predicts
 * that tail from 64 summary features of the alignment with a multilayer
 * perceptron 64 -> 256 -> 256 -> 256 -> 3 (SiLU; BF16 weights, FP32
 * activations and accumulation), trained on the device on fits from
 * simulated nulls.  Its three outputs correct the gamma tail fitted to a few
 * quick nulls (location mu_q, mean excess m_q = tau_q/lambda_q, shape tau_q;
 * features 60-62) towards the tail of many nulls: mu = mu_q + y0 m_q,
 * log(tau/lambda) = log m_q + y1, log tau = log tau_q + y2. */
#define COVGPU_NFEAT 64
#define COVGPU_NOUT 3
#define COVGPU_MLP_NPARAM 148995
#define COVGPU_MLP_MAXMEM 16   /* members of an ensemble */
typedef struct covgpu_mlp covgpu_mlp;

/* the alignment part (features 0-46; 47-63 are set to 0) of the learned
 * null's input for the alignment in slot, with the context's weights:
 * log N, log L, log effective N, pairwise identity (mean, sd), column
 * entropy and gap fraction (mean, sd, 16-bin histograms), residue
 * composition, weight spread and tree_len, the caller's tree-length summary
 * (the mean root-to-leaf length of the alignment's tree) */
int  covgpu_features(covgpu_ctx *ctx, int slot, double tree_len, float *feat);
/* all 64 features of the alignment in slot 0: the alignment part and, in
 * 47-63, a summary of the scores of nquick null alignments of covtype (run
 * as covgpu_rscape with nshuffle = nquick): 47 log of their number; 60-62
 * their tail fit (mu_q, log m_q, log tau_q; m_q the mean excess); and as
 * offsets from mu_q in units of m_q: 48 their mean, 49 their sd, 50-59 the
 * upper quantiles at survival 0.5 ... 0.0005, 63 the largest score */
int  covgpu_learned_features(covgpu_ctx *ctx, const covgpu_params *p, double tree_len, int covtype, int nquick,
                             float *feat);

/* a network with LeCun-uniform weights from seed; batch_cap rows per batch.
 * Parameters are FP32 masters, layer by layer W[out][in] then b[out]. */
int  covgpu_mlp_create(covgpu_mlp **ret, int device, int batch_cap, uint64_t seed);
void covgpu_mlp_destroy(covgpu_mlp *net);
const char *covgpu_mlp_errmsg(const covgpu_mlp *net);
int  covgpu_mlp_set_params(covgpu_mlp *net, const float *params);
int  covgpu_mlp_get_params(covgpu_mlp *net, float *params);
/* inputs x' = (x - xmean)/xstd, outputs y = y' ystd + ymean; features within
 * [xlo, xhi] (may be NULL: unbounded) are inside the training range */
int  covgpu_mlp_set_norm(covgpu_mlp *net, const float *xmean, const float *xstd, const float *ymean,
                         const float *ystd, const float *xlo, const float *xhi);
int  covgpu_mlp_get_norm(const covgpu_mlp *net, float *xmean, float *xstd, float *ymean, float *ystd, float *xlo,
                         float *xhi);
/* an ensemble: nmem parameter sets params[nmem][COVGPU_MLP_NPARAM] (nmem
 * 0..COVGPU_MLP_MAXMEM, 0 = none) sharing this network's standardisation;
 * covgpu_mlp_forward (and so covgpu_rscape_learned) then averages the
 * members' standardised outputs in member order.  Training and gradients
 * keep using the network's own parameters. */
int  covgpu_mlp_set_members(covgpu_mlp *net, const float *params, int nmem);
/* 1 if every feature lies inside the training range */
int  covgpu_mlp_in_range(const covgpu_mlp *net, const float *feat);
/* Y[n][3] = network(X[n][64]) */
int  covgpu_mlp_forward(covgpu_mlp *net, const float *X, int n, float *Y);
/* the mean squared error on standardised targets of one batch of n rows
 * (n <= batch_cap) and its gradient grad[COVGPU_MLP_NPARAM]; no update */
int  covgpu_mlp_grad(covgpu_mlp *net, const float *X, const float *T, int n, float *grad, float *loss);
/* AdamW (beta 0.9/0.999, cosine decay of lr to 5%) over epochs of shuffled
 * batches, each step one replayed CUDA graph; epoch_loss[epochs] (may be NULL) */
int  covgpu_mlp_train(covgpu_mlp *net, const float *X, const float *T, int n, int epochs, int batch, float lr,
                      float wd, uint64_t seed, float *epoch_loss);
/* covgpu_rscape for one covariation type with the learned null: simulates
 * nquick null alignments (instead of p->nshuffle), and when the 64 features
 * are inside the network's training range takes the null tail (mass
 * p->pmass) from the network; otherwise falls back to covgpu_rscape with
 * p->nshuffle simulated nulls.  *used_net tells which.  The result's mu,
 * lambda, tau are the tail used; its nshuffle the nulls simulated. */
int  covgpu_rscape_learned(covgpu_ctx *ctx, const covgpu_params *p, const uint8_t *ax, const double *wgt,
                           covgpu_mlp *net, double tree_len, int covtype, int nquick, covgpu_result *result,
                           covgpu_hit *hits, int hitcap, int *used_net);

/* ---- helix aggregation (agg_CalculatePvalues, src/aggregate.c:41-128) ----
 * covgpu_helices splits a nested consensus structure ct[L] (0-based partner
 * or -1) into helices as R-scape does (ct_split_rmlist,
 * src/structure.c:2990-3142): a pair opens a new helix when it closes a
 * hairpin, a multiloop, or more than helix_unpaired (R-scape: 2) unpaired
 * residues around one inner helix.  Output: *nh helices, helix_off[nh+1]
 * (room for L/2+1), pairs bp_i < bp_j [L/2] grouped by helix, each helix in
 * increasing i.  Host code.  Returns 0, 11 (ct not a pairing) or 13
 * (pseudoknot). */
int  covgpu_helices(const int *ct, int L, int helix_unpaired, int *nh, int *helix_off, int *bp_i, int *bp_j);
/* the aggregated p-value of each helix on the device from the p-values of
 * its pairs, pval[helix_off[nh]] in covgpu_helices order:
 * COVGPU_AGG_FISHER (agg_FISHER, src/aggregate.c:141-176), _LANCASTER
 * (:189-236; aux = the pairs' substitution counts, weights 1 + aux),
 * _WFISHER (:248-289; aux = the pairs' power, weights 0.01 + aux scaled to
 * sum 2 nbp), _SIDAK (:297-322).  A helix of one pair keeps its p-value.
 * Eagg (may be NULL) = nh * pagg.  Chi-square quantiles are taken on the
 * upper tail (Q^-1(w/2, p)), not as the lower-tail inverse at 1 - p. */
enum { COVGPU_AGG_FISHER = 0, COVGPU_AGG_LANCASTER = 1, COVGPU_AGG_WFISHER = 2, COVGPU_AGG_SIDAK = 3 };
int  covgpu_aggregate(covgpu_ctx *ctx, int method, int nh, const int *helix_off, const double *pval,
                      const double *aux, double *pagg, double *Eagg);

/* ---- host utilities for preparing alignments ---- */
/* synthetic RNA alignment: coalescent tree of leaf-to-root length tree_len
 * (Easel convention, arrays of N-1),
 * nbp base pairs in nhelix hairpins of hmin..hmax pairs, gap runs; ct[L] =
 * partner column or -1.  Returns 0 or 11 (bad sizes). */
int  covgpu_synth(int N, int L, double tree_len, int nbp, int nhelix, int hmin, int hmax, double gap_rate,
                  double gap_mean, uint64_t seed, uint8_t *ax, int *parent, int *left, int *right, double *ld,
                  double *rd, int *ct);
/* the same with a choice of tree: 0 = Kingman coalescent (covgpu_synth),
 * 1 = equal waiting times between merges */
int  covgpu_synth2(int N, int L, int tree_kind, double tree_len, int nbp, int nhelix, int hmin, int hmax,
                   double gap_rate, double gap_mean, uint64_t seed, uint8_t *ax, int *parent, int *left, int *right,
                   double *ld, double *rd, int *ct);
/* the rate matrices and backgrounds of covgpu_synth's model (K80 singles,
 * 16-state pair model), for covgpu_simulate */
int  covgpu_synth_model(double *Q4, double *pi4, double *Q16, double *pi16);
/* position-based weights (Henikoff & Henikoff 1994), summing to N */
int  covgpu_weights_pb(const uint8_t *ax, int N, int L, double *wgt);
/* R-scape's gap-column filter: useme[c] = 1 to keep column c */
int  covgpu_gapfilter(const uint8_t *ax, const double *wgt, int N, int L, double gapthresh, int *useme);

#ifdef __cplusplus
}
#endif
#endif
