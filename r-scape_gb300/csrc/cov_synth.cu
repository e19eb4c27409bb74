// cov_synth.cu -- synthetic RNA alignments for benchmarks and tests (host).
//
// Generator of the benchmark workloads: a Kingman coalescent tree with N
// leaves scaled to a leaf-to-root length, helices of base pairs planted as
// hairpins, a root drawn per column, unpaired columns evolved down the tree
// under a 4-state K80/GTR model with equal frequencies and
// transition/transversion ratio 2, paired columns under a reversible
// 16-state pair model with 90% of its stationary mass on the six allowed
// pairs (AU UA CG GC GU UG), and gaps opened per residue with runs of
// geometric length.  Transition matrices P(t) = exp(tQ) per branch are
// formed by scaling and squaring of a Taylor series.  The reference's own
// simulator (src/cov_simulate.c:288-451) plays the same role with a ribosum
// pair model; this one follows the recipe of the benchmark configurations.
// Also position-based sequence weights (Henikoff & Henikoff 1994) and the
// gap-column filter of src/msamanip.c:461-501, host utilities for callers
// that prepare alignments.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "cov_dev.cuh"

using covgpu::philox4x32;

extern "C" int covgpu_synth2(int N, int L, int tree_kind, double tree_len, int nbp, int nhelix, int hmin, int hmax,
                             double gap_rate, double gap_mean, uint64_t seed, uint8_t* ax, int* parent, int* left,
                             int* right, double* ld, double* rd, int* ct);

namespace {

struct Rng {
  uint64_t seed;
  uint32_t stream;
  uint32_t ctr = 0;
  uint32_t buf[4];
  int have = 0;
  uint32_t u32() {
    if (have == 0) {
      uint32_t c[4] = {0x51u, stream, ctr++, 0u};
      philox4x32((uint32_t)seed, (uint32_t)(seed >> 32), c);
      memcpy(buf, c, sizeof(buf));
      have = 4;
    }
    return buf[--have];
  }
  double uni() {  // [0,1)
    const uint64_t a = u32() >> 5, b = u32() >> 6;
    return (double)(a * 67108864ull + b) * (1.0 / 9007199254740992.0);
  }
  double expo(double rate) { return -std::log1p(-uni()) / rate; }
  int below(int n) { return (int)(((uint64_t)u32() * (uint64_t)n) >> 32); }
};

// P = exp(t Q) for an n x n rate matrix, scaling and squaring + Taylor(16)
void expm(const std::vector<double>& Q, int n, double t, std::vector<double>& P) {
  double nrm = 0.0;
  for (int i = 0; i < n; i++) {
    double r = 0.0;
    for (int j = 0; j < n; j++) r += std::fabs(Q[i * n + j]) * t;
    nrm = std::max(nrm, r);
  }
  int sq = 0;
  while (nrm > 0.25) { nrm *= 0.5; sq++; }
  const double scale = t / std::ldexp(1.0, sq);
  std::vector<double> A(n * n), term(n * n), tmp(n * n);
  for (int k = 0; k < n * n; k++) A[k] = Q[k] * scale;
  P.assign(n * n, 0.0);
  for (int i = 0; i < n; i++) P[i * n + i] = 1.0;
  term = P;
  for (int m = 1; m <= 16; m++) {
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        double s = 0.0;
        for (int k = 0; k < n; k++) s += term[i * n + k] * A[k * n + j];
        tmp[i * n + j] = s / m;
      }
    term = tmp;
    for (int k = 0; k < n * n; k++) P[k] += term[k];
  }
  for (int r = 0; r < sq; r++) {
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        double s = 0.0;
        for (int k = 0; k < n; k++) s += P[i * n + k] * P[k * n + j];
        tmp[i * n + j] = s;
      }
    P = tmp;
  }
  for (int i = 0; i < n; i++) {   // clamp rounding negatives, renormalise rows
    double s = 0.0;
    for (int j = 0; j < n; j++) { if (P[i * n + j] < 0.0) P[i * n + j] = 0.0; s += P[i * n + j]; }
    for (int j = 0; j < n; j++) P[i * n + j] /= s;
  }
}

bool is_transition(int a, int b) { return (a == 0 && b == 2) || (a == 2 && b == 0) || (a == 1 && b == 3) || (a == 3 && b == 1); }
bool allowed_pair(int x, int y) {
  return (x == 0 && y == 3) || (x == 3 && y == 0) || (x == 1 && y == 2) || (x == 2 && y == 1) || (x == 2 && y == 3) ||
         (x == 3 && y == 2);
}

void rate4(std::vector<double>& Q) {
  const double kappa = 2.0;
  Q.assign(16, 0.0);
  for (int a = 0; a < 4; a++) {
    double s = 0.0;
    for (int b = 0; b < 4; b++)
      if (a != b) { Q[a * 4 + b] = 0.25 * (is_transition(a, b) ? kappa : 1.0); s += Q[a * 4 + b]; }
    Q[a * 4 + a] = -s;
  }
  double mean = 0.0;
  for (int a = 0; a < 4; a++) mean += 0.25 * -Q[a * 4 + a];
  for (auto& q : Q) q /= mean;
}

void rate16(std::vector<double>& Q, std::vector<double>& pi) {
  const double kappa = 2.0;
  pi.assign(16, 0.0);
  for (int x = 0; x < 4; x++)
    for (int y = 0; y < 4; y++) pi[x * 4 + y] = allowed_pair(x, y) ? 0.15 : 0.01;
  Q.assign(256, 0.0);
  for (int a = 0; a < 16; a++) {
    double s = 0.0;
    for (int b = 0; b < 16; b++) {
      if (a == b) continue;
      const int x = a / 4, y = a % 4, x2 = b / 4, y2 = b % 4;
      double r = 0.0;
      if (x == x2 && y != y2) r = is_transition(y, y2) ? kappa : 1.0;
      if (y == y2 && x != x2) r = is_transition(x, x2) ? kappa : 1.0;
      Q[a * 16 + b] = r * pi[b];
      s += Q[a * 16 + b];
    }
    Q[a * 16 + a] = -s;
  }
  double mean = 0.0;
  for (int a = 0; a < 16; a++) mean += pi[a] * -Q[a * 16 + a];
  for (auto& q : Q) q *= 2.0 / mean;    // two nucleotides per pair
}

int draw(const double* row, int n, double u) {
  double c = 0.0;
  for (int k = 0; k < n; k++) { c += row[k]; if (u < c) return k; }
  return n - 1;
}

}  // namespace

extern "C" int covgpu_synth(int N, int L, double tree_len, int nbp, int nhelix, int hmin, int hmax, double gap_rate,
                            double gap_mean, uint64_t seed, uint8_t* ax, int* parent, int* left, int* right,
                            double* ld, double* rd, int* ct) {
  return covgpu_synth2(N, L, 0, tree_len, nbp, nhelix, hmin, hmax, gap_rate, gap_mean, seed, ax, parent, left, right,
                       ld, rd, ct);
}

// tree_kind 0: Kingman coalescent (exponential waiting times k(k-1)/2);
// tree_kind 1: equal waiting times between merges (every internal branch of
// comparable length, a tree without the long root branches of a coalescent)
extern "C" int covgpu_synth2(int N, int L, int tree_kind, double tree_len, int nbp, int nhelix, int hmin, int hmax,
                             double gap_rate, double gap_mean, uint64_t seed, uint8_t* ax, int* parent, int* left,
                             int* right, double* ld, double* rd, int* ct) {
  if (N < 2 || L < 1 || nbp < 0 || (nbp > 0 && (nhelix < 1 || hmin < 1 || hmax < hmin))) return 11;
  if (tree_kind != 0 && tree_kind != 1) return 11;
  Rng tr{seed, 1}, st{seed, 2}, gp{seed, 3}, ev{seed, 4};
  // ---- random merge tree, internal nodes numbered root = 0, parent < child
  std::vector<int> lineage(N);
  std::vector<double> height(N - 1, 0.0);
  std::vector<int> lch(N - 1), rch(N - 1);
  for (int i = 0; i < N; i++) lineage[i] = -i;      // leaf codes
  double t = 0.0;
  int k = N, m = 0;
  while (k > 1) {
    t += (tree_kind == 0) ? tr.expo(0.5 * k * (k - 1)) : 1.0;
    const int a = tr.below(k);
    int b = tr.below(k - 1);
    if (b >= a) b++;
    const int v = N - 2 - m;
    lch[v] = lineage[a]; rch[v] = lineage[b];
    height[v] = t;
    const int lo = std::min(a, b), hi = std::max(a, b);
    lineage[lo] = v;
    lineage[hi] = lineage[k - 1];
    k--; m++;
  }
  // "total branch length" as R-scape-sim's --atbl: the average leaf-to-root
  // length (src/R-scape-sim.c:84,160,671), i.e. the height of this
  // ultrametric tree
  auto hgt = [&](int c) { return c <= 0 ? 0.0 : height[c]; };
  const double scale = tree_len / height[0];
  for (int v = 0; v < N - 1; v++) {
    left[v] = lch[v]; right[v] = rch[v];
    ld[v] = height[v] - hgt(lch[v]);
    rd[v] = height[v] - hgt(rch[v]);
  }
  parent[0] = -1;
  for (int v = 0; v < N - 1; v++) {
    ld[v] *= scale; rd[v] *= scale;
    if (left[v] > 0) parent[left[v]] = v;
    if (right[v] > 0) parent[right[v]] = v;
  }
  // ---- planted hairpins
  for (int c = 0; c < L; c++) ct[c] = -1;
  if (nbp > 0) {
    std::vector<int> len(nhelix, hmin);
    int rem = nbp - hmin * nhelix;
    if (rem < 0) return 11;
    while (rem > 0) {
      int idx = st.below(nhelix);
      if (len[idx] < hmax) { len[idx]++; rem--; }
      bool full = true;
      for (int h = 0; h < nhelix; h++) if (len[h] < hmax) full = false;
      if (full && rem > 0) return 11;
    }
    int need = 0;
    for (int h = 0; h < nhelix; h++) need += 2 * len[h] + 4;
    if (need > L) return 11;
    const int spare = L - need;
    std::vector<int> gaps(nhelix + 1, 0);
    for (int s = 0; s < spare; s++) gaps[st.below(nhelix + 1)]++;
    int pos = 0;
    for (int h = 0; h < nhelix; h++) {
      pos += gaps[h];
      for (int q = 0; q < len[h]; q++) {
        const int i = pos + q, j = pos + 2 * len[h] + 4 - 1 - q;
        ct[i] = j; ct[j] = i;
      }
      pos += 2 * len[h] + 4;
    }
  }
  // ---- evolve
  std::vector<double> Q4, Q16, pi16;
  rate4(Q4);
  rate16(Q16, pi16);
  const int nn = 2 * N - 1;               // rows: leaves 0..N-1, internal N+v
  std::vector<uint8_t> seq((size_t)nn * L);
  for (int c = 0; c < L; c++) {
    if (ct[c] >= 0 && ct[c] < c) continue;
    if (ct[c] > c) {
      const int s = draw(pi16.data(), 16, ev.uni());
      seq[(size_t)N * L + c] = (uint8_t)(s / 4);
      seq[(size_t)N * L + ct[c]] = (uint8_t)(s % 4);
    } else {
      seq[(size_t)N * L + c] = (uint8_t)ev.below(4);
    }
  }
  std::vector<double> P4, P16;
  for (int v = 0; v < N - 1; v++) {
    const int ch[2] = {left[v], right[v]};
    const double bl[2] = {ld[v], rd[v]};
    for (int s = 0; s < 2; s++) {
      const int row = (ch[s] <= 0) ? -ch[s] : N + ch[s];
      expm(Q4, 4, bl[s], P4);
      expm(Q16, 16, bl[s], P16);
      const uint8_t* pa = &seq[(size_t)(N + v) * L];
      uint8_t* cs = &seq[(size_t)row * L];
      for (int c = 0; c < L; c++) {
        if (ct[c] >= 0 && ct[c] < c) continue;
        if (ct[c] > c) {
          const int a = pa[c] * 4 + pa[ct[c]];
          const int b = draw(&P16[a * 16], 16, ev.uni());
          cs[c] = (uint8_t)(b / 4); cs[ct[c]] = (uint8_t)(b % 4);
        } else {
          cs[c] = (uint8_t)draw(&P4[pa[c] * 4], 4, ev.uni());
        }
      }
    }
  }
  // ---- gaps: runs opened per residue, geometric lengths of mean gap_mean
  const double popen = (gap_mean > 0.0) ? gap_rate / gap_mean : 0.0;
  const double pext = (gap_mean > 1.0) ? 1.0 - 1.0 / gap_mean : 0.0;
  for (int n = 0; n < N; n++) {
    uint8_t* row = &seq[(size_t)n * L];
    int c = 0;
    while (c < L) {
      if (gp.uni() < popen) {
        do { row[c++] = 4; } while (c < L && gp.uni() < pext);
      } else {
        c++;
      }
    }
    memcpy(ax + (size_t)n * L, row, L);
  }
  return 0;
}

extern "C" int covgpu_synth_model(double* Q4, double* pi4, double* Q16, double* pi16) {
  std::vector<double> q4, q16, p16;
  rate4(q4);
  rate16(q16, p16);
  for (int k = 0; k < 16; k++) Q4[k] = q4[k];
  for (int k = 0; k < 4; k++) pi4[k] = 0.25;
  for (int k = 0; k < 256; k++) Q16[k] = q16[k];
  double s = 0.0;
  for (int k = 0; k < 16; k++) s += p16[k];
  for (int k = 0; k < 16; k++) pi16[k] = p16[k] / s;
  return 0;
}

// Henikoff & Henikoff position-based weights over canonical residues,
// renormalised to sum to N (R-scape's choice for nseq > 1000,
// src/R-scape.c:1556)
extern "C" int covgpu_weights_pb(const uint8_t* ax, int N, int L, double* wgt) {
  std::vector<double> w(N, 0.0);
  for (int c = 0; c < L; c++) {
    int cnt[4] = {0, 0, 0, 0}, types = 0;
    for (int s = 0; s < N; s++) { const int x = ax[(size_t)s * L + c]; if (x < 4) cnt[x]++; }
    for (int x = 0; x < 4; x++) if (cnt[x]) types++;
    if (!types) continue;
    for (int s = 0; s < N; s++) {
      const int x = ax[(size_t)s * L + c];
      if (x < 4) w[s] += 1.0 / ((double)types * cnt[x]);
    }
  }
  double sum = 0.0;
  for (double v : w) sum += v;
  for (int s = 0; s < N; s++) wgt[s] = (sum > 0.0) ? w[s] * N / sum : 1.0;
  return 0;
}

// msamanip_RemoveGapColumns (src/msamanip.c:461-501): keep a column iff its
// weighted residue fraction is >= 1 - gapthresh; useme[L] on return
extern "C" int covgpu_gapfilter(const uint8_t* ax, const double* wgt, int N, int L, double gapthresh, int* useme) {
  const double idthresh = 1.0 - gapthresh;
  for (int c = 0; c < L; c++) {
    double r = 0.0, tot = 0.0;
    for (int s = 0; s < N; s++) {
      const int x = ax[(size_t)s * L + c];
      const double w = wgt ? wgt[s] : 1.0;
      if (x < 4 || (x > 4 && x <= 15)) { r += w; tot += w; }
      else if (x == 4 || x == 16) tot += w;
    }
    useme[c] = (r > 0.0 && r / tot >= idthresh) ? 1 : 0;
  }
  return 0;
}
