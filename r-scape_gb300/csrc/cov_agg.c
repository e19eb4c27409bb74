/* cov_agg.c -- the helices of a consensus structure, for helix aggregation.
 *
 * R-scape aggregates the p-values of the base pairs of each helix
 * (agg_CalculatePvalues, src/aggregate.c:41-128) after splitting the
 * structure into helices (struct_rmlist_FromCTLIST -> ct_split_rmlist,
 * src/structure.c:754-793, 2990-3142).  The split is a left-to-right stack
 * scan: unpaired residues and left ends are pushed; at a right end the stack
 * is popped down to its partner, counting the unpaired residues and the
 * closed substructures ("faces") passed on the way.  A pair opens a new
 * helix when it closes a hairpin (no face), a multiloop (more than one face)
 * or, around a single face, more than helix_unpaired unpaired residues;
 * otherwise it joins the helix created last.  Only nested structures are
 * split (the reference rejects pseudoknots here too).
 */
#include <stdlib.h>
#include <string.h>

#include "covgpu.h"

int covgpu_helices(const int *ct, int L, int helix_unpaired, int *ret_nh, int *helix_off, int *bp_i, int *bp_j) {
  if (!ret_nh || L < 0 || (L > 0 && (!ct || !helix_off || !bp_i || !bp_j))) return 11;
  *ret_nh = 0;
  if (L == 0) { helix_off[0] = 0; return 0; }
  for (int j = 0; j < L; j++) {
    const int i = ct[j];
    if (i < -1 || i >= L || i == j || (i >= 0 && ct[i] != j)) return 11;
  }
  int *stack = malloc(sizeof(int) * (2 * (size_t)L + 1));
  int *hid = malloc(sizeof(int) * ((size_t)L / 2 + 1));
  int *pi = malloc(sizeof(int) * ((size_t)L / 2 + 1));
  int *pj = malloc(sizeof(int) * ((size_t)L / 2 + 1));
  int *cnt = calloc((size_t)L / 2 + 2, sizeof(int));
  if (!stack || !hid || !pi || !pj || !cnt) { free(stack); free(hid); free(pi); free(pj); free(cnt); return 5; }
  int sp = 0, nh = 0, nbp = 0, cur = -1, status = 0;
  for (int j = 0; j < L && !status; j++) {
    if (ct[j] < 0 || ct[j] > j) { stack[sp++] = j; continue; }
    const int i = ct[j];
    int nsingle = 0, nfaces = 0, found = 0;
    while (sp > 0) {
      const int v = stack[--sp];
      if (v < 0)       { nfaces++; continue; }     /* a closed substructure */
      if (v == i)      { found = 1; break; }
      if (ct[v] < 0)   { nsingle++; continue; }
      status = 13;                                  /* paired elsewhere: a pseudoknot */
      break;
    }
    if (status) break;
    if (!found) { status = 13; break; }
    if (nfaces == 0 || nfaces > 1 || nsingle > helix_unpaired) cur = nh++;
    stack[sp++] = -1;
    hid[nbp] = cur; pi[nbp] = i; pj[nbp] = j;
    nbp++;
  }
  if (!status) {
    /* pairs grouped by helix, each helix in increasing left end (the
     * reference's pair order, src/aggregate.c:344-354) */
    for (int k = 0; k < nbp; k++) cnt[hid[k] + 1]++;
    for (int h = 0; h < nh; h++) cnt[h + 1] += cnt[h];
    memcpy(helix_off, cnt, sizeof(int) * (size_t)(nh + 1));
    for (int k = 0; k < nbp; k++) {
      const int h = hid[k];
      int q = cnt[h]++;
      /* insertion by left end within the helix */
      while (q > helix_off[h] && bp_i[q - 1] > pi[k]) { bp_i[q] = bp_i[q - 1]; bp_j[q] = bp_j[q - 1]; q--; }
      bp_i[q] = pi[k]; bp_j[q] = pj[k];
    }
    *ret_nh = nh;
  }
  free(stack); free(hid); free(pi); free(pj); free(cnt);
  return status;
}
