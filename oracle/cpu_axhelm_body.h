/* One order of the CPU baseline axhelm; included by cpu_axhelm.c with NQ set.
 * The loop nests restate axhelm/kernel/CPU/axhelm.c (axhelm_v0 :27-111,
 * axhelm_bk_v0 :229-305): per element, q staged in a local cube, the three
 * derivatives and the geometric factors in one sweep, the transposed
 * derivatives in a second, lambda0 = lambda[id], lambda1 = lambda[id+offset]. */
#define NQ2_ (NQ * NQ)
#define NP_ (NQ * NQ * NQ)

static inline __attribute__((always_inline)) void CB_CAT(cb_element_nq, NQ)(
    int bk, int64_t element, int64_t offset, const double (*restrict D)[NQ],
    const double* restrict ggeo, const double* restrict lambda, const double* restrict q,
    double* restrict Aq)
{
  double s_q[NQ][NQ][NQ], s_Gqr[NQ][NQ][NQ], s_Gqs[NQ][NQ][NQ], s_Gqt[NQ][NQ][NQ];
  const int64_t ebase = element * NP_;
  const int64_t gbase = element * 7 * (int64_t)NP_;
  for (int k = 0; k < NQ; ++k)
    for (int j = 0; j < NQ; ++j)
      for (int i = 0; i < NQ; ++i) s_q[k][j][i] = q[ebase + i + j * NQ + k * NQ2_];
  for (int k = 0; k < NQ; ++k)
    for (int j = 0; j < NQ; ++j)
      for (int i = 0; i < NQ; ++i) {
        const int n = i + j * NQ + k * NQ2_;
        const double G00 = ggeo[gbase + 1 * NP_ + n], G01 = ggeo[gbase + 2 * NP_ + n];
        const double G02 = ggeo[gbase + 3 * NP_ + n], G11 = ggeo[gbase + 4 * NP_ + n];
        const double G12 = ggeo[gbase + 5 * NP_ + n], G22 = ggeo[gbase + 6 * NP_ + n];
        double qr = 0, qs = 0, qt = 0;
        for (int m = 0; m < NQ; ++m) {
          qr += D[i][m] * s_q[k][j][m];
          qs += D[j][m] * s_q[k][m][i];
          qt += D[k][m] * s_q[m][j][i];
        }
        double gr = G00 * qr + G01 * qs + G02 * qt;
        double gs = G01 * qr + G11 * qs + G12 * qt;
        double gt = G02 * qr + G12 * qs + G22 * qt;
        if (!bk) {
          const double lam0 = lambda[ebase + n];
          gr *= lam0;
          gs *= lam0;
          gt *= lam0;
        }
        s_Gqr[k][j][i] = gr;
        s_Gqs[k][j][i] = gs;
        s_Gqt[k][j][i] = gt;
      }
  for (int k = 0; k < NQ; ++k)
    for (int j = 0; j < NQ; ++j)
      for (int i = 0; i < NQ; ++i) {
        const int n = i + j * NQ + k * NQ2_;
        double ar = 0, as = 0, at = 0;
        for (int m = 0; m < NQ; ++m) {
          ar += D[m][i] * s_Gqr[k][j][m];
          as += D[m][j] * s_Gqs[k][m][i];
          at += D[m][k] * s_Gqt[m][j][i];
        }
        double out = ar + as + at;
        if (!bk) out += ggeo[gbase + n] * lambda[ebase + n + offset] * s_q[k][j][i];
        Aq[ebase + n] = out;
      }
}

static void CB_CAT(cb_axhelm_nq, NQ)(int bk, int64_t E, int64_t offset,
                                      const double* restrict ggeo, const double* restrict Dg,
                                      const double* restrict lambda, const double* restrict q,
                                      double* restrict Aq)
{
  double D[NQ][NQ];
  for (int j = 0; j < NQ; ++j)
    for (int i = 0; i < NQ; ++i) D[j][i] = Dg[j * NQ + i];
  if (bk) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; ++e)
      CB_CAT(cb_element_nq, NQ)(1, e, offset, (const double(*)[NQ])D, ggeo, lambda, q, Aq);
  } else {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; ++e)
      CB_CAT(cb_element_nq, NQ)(0, e, offset, (const double(*)[NQ])D, ggeo, lambda, q, Aq);
  }
}

#undef NQ2_
#undef NP_
