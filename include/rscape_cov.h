/* rscape_cov.h -- drop-in C entry points of R-scape's covariation path,
 * backed by the GB300 engine (libcovgpu.so).
 *
 * Each function keeps the name, argument meaning and int-status/errbuf error
 * convention of the reference declaration it replaces:
 *   correlators.h  src/correlators.h:445-482
 *   covariation.h  src/covariation.h:27-60
 * The Easel types the reference passes (ESL_MSA, ESL_DMATRIX, ESL_HISTOGRAM,
 * ESL_TREE, ESL_ALPHABET, ESL_RANDOMNESS) appear here as layout-defined shims
 * holding the fields the covariation path reads; R-scape's own structs
 * (struct mutual_s, struct data_s, RANKLIST, HIT, HITLIST, THRESH) keep the
 * fields of src/correlators.h:107-177, 374-442 that this path uses.  A build
 * of R-scape against real Easel headers maps its objects onto these shims
 * field by field (see the integration notes shipped with the library).
 */
#ifndef RSCAPE_COV_H
#define RSCAPE_COV_H
#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- Easel shims ---------------- */
#define eslOK      0
#define eslFAIL    1
#define eslEMEM    5
#define eslEINVAL 11
#define eslERANGE 19

#define eslRNA 1
#define eslDNA 2

typedef uint8_t ESL_DSQ;

typedef struct {
  int type;        /* eslRNA */
  int K;           /* 4 canonical residues */
  int Kp;          /* 18 codes: ACGU-RYMKSWHBVDN*~ */
} ESL_ALPHABET;

typedef struct {
  ESL_DSQ           **ax;    /* digital rows, residues at ax[s][1..alen] */
  double             *wgt;   /* sequence weights [nseq] */
  int                 nseq;
  int64_t             alen;
  const ESL_ALPHABET *abc;
} ESL_MSA;

typedef struct {
  double **mx;     /* mx[i][j] */
  int      n, m;
} ESL_DMATRIX;

typedef struct {
  double    xmin, xmax;   /* smallest, largest sample value */
  uint64_t  n;            /* number of samples */
  uint64_t *obs;          /* observed counts in bin b, 0..nb-1 */
  double    bmin, bmax;   /* histogram bounds */
  double    w;            /* bin width */
  int       imin, imax;   /* smallest, largest bin with data */
  int       nb;           /* number of bins */
  double    phi;          /* censoring / tail threshold */
  int       cmin;         /* smallest bin in the fitted tail */
  uint64_t  Nc;           /* total count including censored data */
  uint64_t  No;           /* count in the fitted tail */
} ESL_HISTOGRAM;

typedef struct {
  int     N;              /* leaves */
  int    *parent;         /* [N-1] */
  int    *left, *right;   /* [N-1]: > 0 internal node, <= 0 leaf -value */
  double *ld, *rd;        /* [N-1] branch lengths */
} ESL_TREE;

typedef struct {
  uint64_t seed;          /* counter-based streams are keyed by this seed */
} ESL_RANDOMNESS;

/* ---------------- R-scape types (src/correlators.h) ---------------- */
typedef enum { C16 = 0, C2 = 1, CWC = 2, CSELECT = 3 } COVCLASS;
typedef enum {
  CHI = 0, CHIp = 1, CHIa = 2, GT = 3, GTp = 4, GTa = 5, MI = 6, MIp = 7, MIa = 8,
  MIr = 9, MIrp = 10, MIra = 11, MIg = 12, MIgp = 13, MIga = 14, OMES = 15, OMESp = 16, OMESa = 17,
  RAF = 18, RAFp = 19, RAFa = 20, RAFS = 21, RAFSp = 22, RAFSa = 23, CCF = 24, CCFp = 25, CCFa = 26,
  PTFp = 27, PTAp = 28, PTDp = 29, COVNONE = 30
} COVTYPE;
typedef enum { APC = 0, ASC = 1 } ACTYPE;
typedef enum { NONPARAM = 0, POTTS = 1, AKMAEV = 2 } METHOD;
typedef enum { NAIVE = 0, NULLPHYLO = 1, GIVENNULL = 2 } STATSMETHOD;
typedef enum { GIVSS = 0, FOLDSS = 1, RANSS = 2 } MODE;
typedef enum { SAMPLE_CONTACTS = 0, SAMPLE_BP = 1, SAMPLE_WC = 2, SAMPLE_ALL = 3 } SAMPLESIZE;
typedef enum { Eval = 0 } THRESHTYPE;
/* contact types (BPTYPE, lib/R-view/src/rview_contacts.h:22-62): the 32
 * base-pair families 0..31 (WWc = 0), then these three */
typedef enum { WWc = 0, STACKED = 32, CONTACT = 33, BPNONE = 34 } BPTYPE;

/* the fields of CNT and CLIST (rview_contacts.h:65-110) read on this path:
 * contact h joins alignment positions cnt[h].i < cnt[h].j (1-based) */
typedef struct cnt_s {
  int64_t i, j;
  BPTYPE  bptype;
} CNT;
typedef struct clist_s {
  int   ncnt;
  int   mind;     /* with msa2pdb: pairs closer than mind in the PDB are not ranked */
  CNT  *cnt;
} CLIST;

struct mutual_s {
  int64_t       alen;
  int64_t       nseq;
  double     ***pp;        /* [alen][alen][K*K] */
  double      **pm;        /* [alen][K] */
  double      **nseff;     /* [alen][alen] */
  double      **ps;        /* [alen][K+1] */
  double      **ngap;      /* [alen][alen] */
  COVTYPE       type;
  COVCLASS      class_;    /* "class" in the reference (a C++ keyword) */
  ESL_DMATRIX  *COV;
  ESL_DMATRIX  *Eval;
  double        besthreshCOV;
  double        minCOV;
  double        maxCOV;
  int           ishuffled;
  int           nseqthresh;
  int           alenthresh;
  const ESL_ALPHABET *abc;
  void         *gpu;       /* engine state of this object (library-owned) */
  int           device_resident;   /* 0 (corr_Create's default): every call leaves the reference's
                                    * host arrays filled, as R-scape expects.  1: pp, nseff and ngap
                                    * stay on the device (corr_ValidateProbs checks them there), and
                                    * COV and Eval stay on the device from corr_Calculate* through
                                    * corr_CalculateCOVCorrected, cov_SignificantPairs_Ranking and
                                    * cov_CreateHitList (the hit list and minCOV/maxCOV come back);
                                    * corr_SyncHost copies COV to the host.  A caller sets it after
                                    * corr_Create when nothing reads those arrays (no power
                                    * analysis, no CaCoFold), and must not write mi->COV meanwhile.
                                    * With 0, a shuffled alignment (ishuffled, R-scape's nulls) is
                                    * treated as with 1: R-scape reads only its ranklist and
                                    * minCOV/maxCOV, and the host arrays keep the last given
                                    * alignment's values. */
};

typedef struct ranklist_s {
  ESL_HISTOGRAM *ha;       /* all pairs */
  ESL_HISTOGRAM *ht;       /* pairs outside the given structure */
  ESL_HISTOGRAM *hb;       /* base pairs of the given structure */
  double        *survfit;
} RANKLIST;

typedef struct hit_s {
  int64_t i, j;
  double  sc, Eval, pval;
  int64_t nsubs;
  double  power;
  int     bptype;
  int     is_compatible;
} HIT;

typedef struct hitlist_s {
  int      nhit;
  HIT    **srthit;
  HIT     *hit;
  int64_t  Nt;
  int64_t  Nb;
} HITLIST;

typedef struct thresh_s {
  THRESHTYPE type;
  double     val;
  double     sc_bp;
  double     sc_nbp;
} THRESH;

typedef struct RMlist_s RMLIST;   /* helix aggregation: outside this library */

/* the fields of struct data_s (src/correlators.h:374-442) read on this path */
struct data_s {
  ESL_RANDOMNESS  *r;
  SAMPLESIZE       samplesize;
  RANKLIST        *ranklist_null;
  RANKLIST        *ranklist_aux;
  struct mutual_s *mi;
  THRESH          *thresh;
  STATSMETHOD      statsmethod;
  METHOD           covmethod;
  MODE             mode;
  COVTYPE          covtype;
  int              nseq;
  double           expBP;
  double           bmin;
  double           w;
  double           fracfit;
  double           pmass;
  int              doexpfit;
  double           tau, mu, lambda;
  ESL_DMATRIX     *allowpair;
  double           tol;
  int              verbose;
  char            *errbuf;       /* caller-provided, >= 256 bytes */
  CLIST           *clist;        /* the given structure's contacts (may be NULL: none) */
  int             *msa2pdb;      /* [alen] PDB position of each column, -1 for none (may be NULL) */
};

#define MAX_EVAL 1000

/* ---------------- correlators.h (src/correlators.h:445-482) ---------------- */
extern int  corr_CalculateCHI     (COVCLASS covclass, struct data_s *data);
extern int  corr_CalculateCHI_C16 (struct mutual_s *mi, int verbose, char *errbuf);
extern int  corr_CalculateCHI_C2  (struct mutual_s *mi, ESL_DMATRIX *allowpair, int verbose, char *errbuf);
extern int  corr_CalculateOMES    (COVCLASS covclass, struct data_s *data);
extern int  corr_CalculateOMES_C16(struct mutual_s *mi, int verbose, char *errbuf);
extern int  corr_CalculateOMES_C2 (struct mutual_s *mi, ESL_DMATRIX *allowpair, int verbose, char *errbuf);
extern int  corr_CalculateGT      (COVCLASS covclass, struct data_s *data);
extern int  corr_CalculateGT_C16  (struct mutual_s *mi, int verbose, char *errbuf);
extern int  corr_CalculateGT_C2   (struct mutual_s *mi, ESL_DMATRIX *allowpair, int verbose, char *errbuf);
extern int  corr_CalculateGT_CWC  (struct mutual_s *mi, ESL_DMATRIX *allowpair, int verbose, char *errbuf);
extern int  corr_CalculateMI      (COVCLASS covclass, struct data_s *data);
extern int  corr_CalculateMI_C16  (struct mutual_s *mi, int verbose, char *errbuf);
extern int  corr_CalculateMI_C2   (struct mutual_s *mi, ESL_DMATRIX *allowpair, int verbose, char *errbuf);
extern int  corr_CalculateMIr     (COVCLASS covclass, struct data_s *data);
extern int  corr_CalculateMIr_C16 (struct mutual_s *mi, int verbose, char *errbuf);
extern int  corr_CalculateMIr_C2  (struct mutual_s *mi, ESL_DMATRIX *allowpair, int verbose, char *errbuf);
extern int  corr_CalculateMIg     (COVCLASS covclass, struct data_s *data);
extern int  corr_CalculateMIg_C16 (struct mutual_s *mi, int verbose, char *errbuf);
extern int  corr_CalculateMIg_C2  (struct mutual_s *mi, ESL_DMATRIX *allowpair, int verbose, char *errbuf);
extern int  corr_CalculateRAF     (COVCLASS covclass, struct data_s *data, ESL_MSA *msa);
extern int  corr_CalculateRAFS    (COVCLASS covclass, struct data_s *data, ESL_MSA *msa);
extern int  corr_CalculateCCF     (COVCLASS covclass, struct data_s *data);
extern int  corr_CalculateCCF_C16 (struct mutual_s *mi, int verbose, char *errbuf);
extern int  corr_CalculateCOVCorrected(ACTYPE actype, struct data_s *data, int shiftnonneg);
extern struct mutual_s *corr_Create(int64_t alen, int64_t nseq, int isshuffled, int nseqthresh, int alenthresh,
                                    const ESL_ALPHABET *abc, COVCLASS covclass);
extern int  corr_Reuse(struct mutual_s *mi, int ishuffled, COVTYPE mitype, COVCLASS miclass);
extern int  corr_ReuseCOV(struct mutual_s *mi, COVTYPE mitype, COVCLASS covclass);
extern void corr_Destroy(struct mutual_s *mi);
extern int  corr_NaivePP(ESL_RANDOMNESS *r, ESL_MSA *msa, struct mutual_s *mi, double tol, int verbose, char *errbuf);
extern int  corr_NaivePS(ESL_RANDOMNESS *r, ESL_MSA *msa, struct mutual_s *mi, double tol, int verbose, char *errbuf);
extern int  corr_Marginals(struct mutual_s *mi, double tol, int verbose, char *errbuf);
extern int  corr_Probs(ESL_RANDOMNESS *r, ESL_MSA *msa, ESL_TREE *T, void *ribosum, struct mutual_s *mi,
                       METHOD method, double tol, int verbose, char *errbuf);
extern int  corr_ValidateProbs(struct mutual_s *mi, double tol, int verbose, char *errbuf);
extern int  corr_COVTYPEString(char **ret_covtype, COVTYPE type, char *errbuf);
/* No counterpart in the reference: when the device alone holds the current score matrix
 * (device-resident mode, or a shuffled alignment's scores), copies it into mi->COV (both
 * triangles, diagonal -inf); a no-op otherwise. */
extern int  corr_SyncHost(struct mutual_s *mi, char *errbuf);
extern int  corr_String2COVTYPE(char *covtype, COVTYPE *ret_type, char *errbuf);
/* the Akmaev pair probabilities are not provided: returns eslFAIL (errbuf set) */
extern int  corr_PostOrderPP(ESL_MSA *msa, ESL_TREE *T, void *ribosum, struct mutual_s *mi, double tol, int verbose,
                             char *errbuf);

/* ---------------- covariation.h (src/covariation.h:27-60) ---------------- */
#define BMIN  -10.0
#define HPTS  400
#define W     0.05

extern int       cov_Calculate(struct data_s *data, ESL_MSA *msa, RANKLIST **ret_ranklist, HITLIST **ret_hitlist,
                               RMLIST **ret_rmlist, int analyze);
extern int       cov_SignificantPairs_Ranking(struct data_s *data, RANKLIST **ret_ranklist, HITLIST **ret_hitlist,
                                              RMLIST **ret_rmlist);
extern RANKLIST *cov_CreateRankList(double bmax, double bmin, double w);
extern int       cov_GrowRankList(RANKLIST **oranklist, double bmax, double bmin);
extern int       cov_CreateHitList(struct data_s *data, struct mutual_s *mi, RANKLIST *ranklist, HITLIST **ret_hitlist,
                                   RMLIST **ret_rmlist, char *covtype, char *threshtype);
extern int       cov_ReadNullHistogram(char *nullhisfile, RANKLIST **ret_ranklist, char *errbuf, int verbose);
extern int       cov_WriteNullHistogram(char *nullhisfile, RANKLIST *ranklist, char *errbuf, int verbose);
extern void      cov_FreeRankList(RANKLIST *ranklist);
extern void      cov_FreeHitList(HITLIST *hitlist);
extern int       cov_NullFitGamma(ESL_HISTOGRAM *h, double **ret_survfit, double pmass, double *ret_newmass,
                                  double *ret_mu, double *ret_lambda, double *ret_k, int verbose, char *errbuf);
extern int       cov_NullFitExponential(ESL_HISTOGRAM *h, double **ret_survfit, double pmass, double *ret_newmass,
                                        double *ret_mu, double *ret_lambda, int verbose, char *errbuf);
extern int       cov_histogram_SetSurvFitTail(ESL_HISTOGRAM *h, double **ret_survfit, double pmass,
                                              double (*surv)(double x, void *params), void *params);
extern int       cov_ranklist_Bin2Bin(int b, ESL_HISTOGRAM *h, ESL_HISTOGRAM *new_, int *ret_newb);
extern int       cov_THRESHTYPEString(char **ret_threshtype, THRESHTYPE type, char *errbuf);
extern int       cov_Add2SubsHistogram(ESL_HISTOGRAM *hsubs, HITLIST *hitlist, int verbose);
/* as the reference, both print to stdout whatever fp is */
extern int       cov_DumpRankList(FILE *fp, RANKLIST *ranklist);
extern int       cov_DumpHistogram(FILE *fp, ESL_HISTOGRAM *h);
extern int       cov_SignificantPairs_ZScore(struct mutual_s *mi, int *msamap, int firstpos, int *ct, int verbose,
                                             char *errbuf);
extern int       cov_FisherExactTest(double *ret_pval, int cBP, int cNBP, int BP, int alen);
extern int       cov_histogram_PlotSurvival(FILE *fp, ESL_HISTOGRAM *h, double *survfit);
/* writes covhisfile's survival curves; the gnuplot figures are not drawn
 * (gnuplot, covqqfile and title are not read) */
extern int       cov_WriteHistogram(struct data_s *data, char *gnuplot, char *covhisfile, char *covqqfile,
                                    SAMPLESIZE samplesize, RANKLIST *ranklist, char *title);
/* CaCoFold's hit list is not provided: returns eslFAIL (errbuf set) */
extern int       cov_CreateFOLDHitList(struct data_s *data, void *foldctlist, RANKLIST *ranklist, HITLIST *hitlist,
                                       void *r3d, HITLIST **ret_foldhitlist, RMLIST **ret_foldrmlist, char *covtype,
                                       char *threshtype);

/* ---------------- histogram helpers (Easel esl_histogram restated) ---------------- */
extern ESL_HISTOGRAM *covh_Create(double bmin, double bmax, double w);
extern void           covh_Destroy(ESL_HISTOGRAM *h);
extern int            covh_Score2Bin(const ESL_HISTOGRAM *h, double x, int *ret_b);
extern double         covh_Bin2LBound(const ESL_HISTOGRAM *h, int b);
extern double         covh_Bin2UBound(const ESL_HISTOGRAM *h, int b);
extern int            covh_Add(ESL_HISTOGRAM *h, double x);
extern double         covh_pmass(const ESL_HISTOGRAM *h, double target_pmass, double target_fracfit);
extern double         covh_SetTailByMass(ESL_HISTOGRAM *h, double pmass);   /* returns the tail's mass */
extern double         covh_cov2evalue(double cov, double Nc, const ESL_HISTOGRAM *h, const double *survfit);
extern double         covh_evalue2cov(double eval_thresh, double Nc, const ESL_HISTOGRAM *h, const double *survfit);
extern double         covh_gamma_surv(double x, void *params);   /* params = {mu, lambda, tau} */
extern double         covh_exp_surv(double x, void *params);     /* params = {mu, lambda} */

#ifdef __cplusplus
}
#endif
#endif
