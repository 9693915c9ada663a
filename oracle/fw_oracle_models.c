/*
 * fw_oracle_models.c -- CPU restatement of the detailed ionic models of the
 * reference: ten Tusscher-Panfilov 2006 (TP06) and Courtemanche 1998.
 *
 * TEST INFRASTRUCTURE ONLY (part of the oracle; see fw_oracle.c).
 *
 * Each expression keeps the reference's evaluation order (Python's
 * left-to-right associativity made explicit by its syntax tree); exp, log,
 * sqrt and pow are the C library's, as the reference's numba JIT calls them.
 * `x**2` is x*x as numba compiles it.  The reference's quirks are kept:
 * TP06's Ca_i is never updated (tp06_2d.py:1098 assigns the new value and
 * then the old one), Courtemanche's IKr conductance is fixed at 0.0294 inside
 * calc_ikr (courtemanche_2d.py:420-422) and its run_ionic_kernel hands the
 * model's `xr` array to the kernel's `xs` argument and vice versa
 * (courtemanche_2d.py:152-160 against :581), so the model's `xs` holds the
 * IKr gate and `xr` the IKs gate.
 */
#include <math.h>
#include <stdint.h>

#define EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------ TP06 */
/* Parameter order (ionic_kernel_2d signature, tp06_2d.py:1003-1012). */
enum {
    T_ko, T_cao, T_nao, T_Vc, T_Vsr, T_Vss, T_Bufc, T_Kbufc, T_Bufsr,
    T_Kbufsr, T_Bufss, T_Kbufss, T_Vmaxup, T_Kup, T_Vrel, T_k1_, T_k2_, T_k3,
    T_k4, T_EC, T_maxsr, T_minsr, T_Vleak, T_Vxfer, T_R, T_F, T_T, T_RTONF,
    T_CAPACITANCE, T_gkr, T_pKNa, T_gk1, T_gna, T_gbna, T_KmK, T_KmNa,
    T_knak, T_gcal, T_gbca, T_knaca, T_KmNai, T_KmCa, T_ksat, T_n_, T_gpca,
    T_KpCa, T_gpk, T_gto, T_gks, T_NP
};
/* State order (TP062D.state_vars minus u, tp06_2d.py:77-79). */
enum {
    S_cai, S_casr, S_cass, S_nai, S_Ki, S_m, S_h, S_j, S_xr1, S_xr2, S_xs,
    S_r, S_s, S_d, S_f, S_f2, S_fcass, S_rr, S_oo, S_NS
};

/* TP06 ionic_kernel_2d and the calc_* helpers (cpuwave2D/model/tp06_2d.py:
 * 242-1103; the 3D kernel tp06_3d.py:85-204 is the same per node). */
EXPORT void fwo_ionic_tp06(double *un, const double *u, double *const *S,
                           const int64_t *idx, int64_t n_idx, double dt,
                           const double *P)
{
    const double ko = P[T_ko], cao = P[T_cao], nao = P[T_nao], Vc = P[T_Vc],
                 Vsr = P[T_Vsr], Vss = P[T_Vss], Bufc = P[T_Bufc],
                 Kbufc = P[T_Kbufc], Bufsr = P[T_Bufsr], Kbufsr = P[T_Kbufsr],
                 Bufss = P[T_Bufss], Kbufss = P[T_Kbufss],
                 Vmaxup = P[T_Vmaxup], Kup = P[T_Kup], Vrel = P[T_Vrel],
                 k1 = P[T_k1_], k2 = P[T_k2_], k3 = P[T_k3], k4 = P[T_k4],
                 EC = P[T_EC], maxsr = P[T_maxsr], minsr = P[T_minsr],
                 Vleak = P[T_Vleak], Vxfer = P[T_Vxfer], R = P[T_R],
                 F = P[T_F], T = P[T_T], RTONF = P[T_RTONF],
                 CAP = P[T_CAPACITANCE], gkr = P[T_gkr], pKNa = P[T_pKNa],
                 gk1 = P[T_gk1], gna = P[T_gna], gbna = P[T_gbna],
                 KmK = P[T_KmK], KmNa = P[T_KmNa], knak = P[T_knak],
                 gcal = P[T_gcal], gbca = P[T_gbca], knaca = P[T_knaca],
                 KmNai = P[T_KmNai], KmCa = P[T_KmCa], ksat = P[T_ksat],
                 n_ = P[T_n_], gpca = P[T_gpca], KpCa = P[T_KpCa],
                 gpk = P[T_gpk], gto = P[T_gto], gks = P[T_gks];
    const double inverseVcF2 = 1.0 / (2 * Vc * F);
    const double inverseVcF = 1.0 / (Vc * F);
    const double inversevssF2 = 1.0 / (2 * Vss * F);
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_idx; ++t) {
        const int64_t p = idx[t];
        const double uu = u[p];
        double cai = S[S_cai][p], casr = S[S_casr][p], cass = S[S_cass][p],
               nai = S[S_nai][p], Ki = S[S_Ki][p];
        double m = S[S_m][p], h = S[S_h][p], j = S[S_j][p];
        double xr1 = S[S_xr1][p], xr2 = S[S_xr2][p], xs = S[S_xs][p];
        double r = S[S_r][p], s = S[S_s][p], d = S[S_d][p], f = S[S_f][p],
               f2 = S[S_f2][p], fcass = S[S_fcass][p], rr = S[S_rr][p];

        const double Ek = RTONF * log(ko / Ki);
        const double Ena = RTONF * log(nao / nai);
        const double Eks = RTONF * log((ko + pKNa * nao) / (Ki + pKNa * nai));
        const double Eca = 0.5 * RTONF * log(cao / cai);

        /* calc_ina (tp06_2d.py:242-310) */
        double ina;
        {
            const double alpha_m = 1.0 / (1.0 + exp((-60.0 - uu) / 5.0));
            const double beta_m = 0.1 / (1.0 + exp((uu + 35.0) / 5.0)) +
                                  0.1 / (1.0 + exp((uu - 50.0) / 200.0));
            const double tau_m = alpha_m * beta_m;
            const double m_inf = 1.0 / ((1.0 + exp((-56.86 - uu) / 9.03)) *
                                        (1.0 + exp((-56.86 - uu) / 9.03)));
            double alpha_h, beta_h;
            if (uu >= -40.0) {
                alpha_h = 0.0;
                beta_h = 0.77 / (0.13 * (1.0 + exp(-(uu + 10.66) / 11.1)));
            } else {
                alpha_h = 0.057 * exp(-(uu + 80.0) / 6.8);
                beta_h = 2.7 * exp(0.079 * uu) + 310000.0 * exp(0.3485 * uu);
            }
            const double tau_h = 1.0 / (alpha_h + beta_h);
            const double h_inf = 1.0 / ((1.0 + exp((uu + 71.55) / 7.43)) *
                                        (1.0 + exp((uu + 71.55) / 7.43)));
            double alpha_j, beta_j;
            if (uu >= -40.0) {
                alpha_j = 0.0;
                beta_j = 0.6 * exp(0.057 * uu) / (1.0 + exp(-0.1 * (uu + 32.0)));
            } else {
                alpha_j = (-25428.0 * exp(0.2444 * uu) -
                           6.948e-06 * exp(-0.04391 * uu)) *
                          (uu + 37.78) / (1.0 + exp(0.311 * (uu + 79.23)));
                beta_j = 0.02424 * exp(-0.01052 * uu) /
                         (1.0 + exp(-0.1378 * (uu + 40.14)));
            }
            const double tau_j = 1.0 / (alpha_j + beta_j);
            const double j_inf = h_inf;
            m = m_inf - (m_inf - m) * exp(-dt / tau_m);
            h = h_inf - (h_inf - h) * exp(-dt / tau_h);
            j = j_inf - (j_inf - j) * exp(-dt / tau_j);
            ina = gna * m * m * m * h * j * (uu - Ena);
        }
        /* calc_ical (:313-376) */
        double ical;
        {
            const double d_inf = 1.0 / (1.0 + exp((-8 - uu) / 7.5));
            const double Ad = 1.4 / (1.0 + exp((-35 - uu) / 13)) + 0.25;
            const double Bd = 1.4 / (1.0 + exp((uu + 5) / 5));
            const double Cd = 1.0 / (1.0 + exp((50 - uu) / 20));
            const double tau_d = Ad * Bd + Cd;
            const double f_inf = 1.0 / (1.0 + exp((uu + 20) / 7));
            const double Af = 1102.5 * exp(-(uu + 27) * (uu + 27) / 225);
            const double Bf = 200.0 / (1 + exp((13 - uu) / 10.0));
            const double Cf = 180.0 / (1 + exp((uu + 30) / 10)) + 20;
            const double tau_f = Af + Bf + Cf;
            const double f2_inf = 0.67 / (1.0 + exp((uu + 35) / 7)) + 0.33;
            const double Af2 = 600 * exp(-(uu + 25) * (uu + 25) / 170);
            const double Bf2 = 31 / (1.0 + exp((25 - uu) / 10));
            const double Cf2 = 16 / (1.0 + exp((uu + 30) / 10));
            const double tau_f2 = Af2 + Bf2 + Cf2;
            const double fcass_inf =
                0.6 / (1 + cass / 0.05 * (cass / 0.05)) + 0.4;
            const double tau_fcass =
                80.0 / (1 + cass / 0.05 * (cass / 0.05)) + 2.0;
            d = d_inf - (d_inf - d) * exp(-dt / tau_d);
            f = f_inf - (f_inf - f) * exp(-dt / tau_f);
            f2 = f2_inf - (f2_inf - f2) * exp(-dt / tau_f2);
            fcass = fcass_inf - (fcass_inf - fcass) * exp(-dt / tau_fcass);
            ical = gcal * d * f * f2 * fcass * 4 * (uu - 15) * (F * F / (R * T)) *
                   (0.25 * exp(2 * (uu - 15) * F / (R * T)) * cass - cao) /
                   (exp(2 * (uu - 15) * F / (R * T)) - 1.0);
        }
        /* calc_ito (:379-410) */
        double ito;
        {
            const double r_inf = 1.0 / (1.0 + exp((20 - uu) / 6.0));
            const double s_inf = 1.0 / (1.0 + exp((uu + 20) / 5.0));
            const double tau_r =
                9.5 * exp(-(uu + 40.0) * (uu + 40.0) / 1800.0) + 0.8;
            const double tau_s =
                85.0 * exp(-(uu + 45.0) * (uu + 45.0) / 320.0) +
                5.0 / (1.0 + exp((uu - 20.0) / 5.0)) + 3.0;
            s = s_inf - (s_inf - s) * exp(-dt / tau_s);
            r = r_inf - (r_inf - r) * exp(-dt / tau_r);
            ito = gto * r * s * (uu - Ek);
        }
        /* calc_ikr (:413-450) */
        double ikr;
        {
            const double xr1_inf = 1.0 / (1.0 + exp((-26.0 - uu) / 7.0));
            const double axr1 = 450.0 / (1.0 + exp((-45.0 - uu) / 10.0));
            const double bxr1 = 6.0 / (1.0 + exp((uu - -30.0) / 11.5));
            const double tau_xr1 = axr1 * bxr1;
            const double xr2_inf = 1.0 / (1.0 + exp((uu - -88.0) / 24.0));
            const double axr2 = 3.0 / (1.0 + exp((-60.0 - uu) / 20.0));
            const double bxr2 = 1.12 / (1.0 + exp((uu - 60.0) / 20.0));
            const double tau_xr2 = axr2 * bxr2;
            xr1 = xr1_inf - (xr1_inf - xr1) * exp(-dt / tau_xr1);
            xr2 = xr2_inf - (xr2_inf - xr2) * exp(-dt / tau_xr2);
            ikr = gkr * sqrt(ko / 5.4) * xr1 * xr2 * (uu - Ek);
        }
        /* calc_iks (:453-484) */
        double iks;
        {
            double xs_inf = 1.0 / (1.0 + exp((-5.0 - uu) / 14.0));
            const double Axs = 1400.0 / sqrt(1.0 + exp((5.0 - uu) / 6));
            const double Bxs = 1.0 / (1.0 + exp((uu - 35.0) / 15.0));
            const double tau_xs = Axs * Bxs + 80;
            xs_inf = 1.0 / (1.0 + exp((-5.0 - uu) / 14.0));
            xs = xs_inf - (xs_inf - xs) * exp(-dt / tau_xs);
            iks = gks * xs * xs * (uu - Eks);
        }
        /* calc_ik1 (:487-510) */
        const double ak1 = 0.1 / (1.0 + exp(0.06 * (uu - Ek - 200)));
        const double bk1 = (3.0 * exp(0.0002 * (uu - Ek + 100)) +
                            exp(0.1 * (uu - Ek - 10))) /
                           (1.0 + exp(-0.5 * (uu - Ek)));
        const double rec_iK1 = ak1 / (ak1 + bk1);
        const double ik1 = gk1 * rec_iK1 * (uu - Ek);
        /* calc_inaca (:513-556) */
        const double inaca =
            knaca * (1.0 / (KmNai * KmNai * KmNai + nao * nao * nao)) *
            (1.0 / (KmCa + cao)) *
            (1.0 / (1 + ksat * exp((n_ - 1) * uu * F / (R * T)))) *
            (exp(n_ * uu * F / (R * T)) * nai * nai * nai * cao -
             exp((n_ - 1) * uu * F / (R * T)) * nao * nao * nao * cai * 2.5);
        /* calc_inak (:559-591) */
        const double rec_iNaK =
            1.0 / (1.0 + 0.1245 * exp(-0.1 * uu * F / (R * T)) +
                   0.0353 * exp(-uu * F / (R * T)));
        const double inak =
            knak * (ko / (ko + KmK)) * (nai / (nai + KmNa)) * rec_iNaK;
        /* calc_ipca, calc_ipk, calc_ibna, calc_ibca (:594-680) */
        const double ipca = gpca * cai / (KpCa + cai);
        const double rec_ipK = 1.0 / (1.0 + exp((25 - uu) / 5.98));
        const double ipk = gpk * rec_ipK * (uu - Ek);
        const double ibna = gbna * (uu - Ena);
        const double ibca = gbca * (uu - Eca);
        /* calc_irel (:683-736) */
        const double kCaSR =
            maxsr - (maxsr - minsr) / (1 + EC / casr * (EC / casr));
        const double k1_ = k1 / kCaSR;
        const double k2_ = k2 * kCaSR;
        const double drr = k4 * (1 - rr) - k2_ * cass * rr;
        rr += dt * drr;
        const double oo = k1_ * cass * cass * rr / (k3 + k1_ * cass * cass);
        const double irel = Vrel * oo * (casr - cass);
        /* calc_ileak, calc_iup, calc_ixfer (:739-790) */
        const double ileak = Vleak * (casr - cai);
        const double iup = Vmaxup / (1.0 + Kup * Kup / (cai * cai));
        const double ixfer = Vxfer * (cass - cai);
        /* calc_casr (:793-829) */
        {
            const double CaCSQN = Bufsr * casr / (casr + Kbufsr);
            const double dCaSR = dt * (iup - irel - ileak);
            const double bjsr = Bufsr - CaCSQN - dCaSR - casr + Kbufsr;
            const double cjsr = Kbufsr * (CaCSQN + dCaSR + casr);
            casr = (sqrt(bjsr * bjsr + 4 * cjsr) - bjsr) / 2;
        }
        /* calc_cass (:832-873) */
        {
            const double CaSSBuf = Bufss * cass / (cass + Kbufss);
            const double dCaSS =
                dt * (-ixfer * (Vc / Vss) + irel * (Vsr / Vss) +
                      -ical * inversevssF2 * CAP);
            const double bcss = Bufss - CaSSBuf - dCaSS - cass + Kbufss;
            const double ccss = Kbufss * (CaSSBuf + dCaSS + cass);
            cass = (sqrt(bcss * bcss + 4 * ccss) - bcss) / 2;
        }
        /* calc_cai (:876-921): computed and discarded by the reference's
         * double assignment (tp06_2d.py:1098) -- cai keeps its value. */
        /* calc_nai, calc_ki (:924-966) */
        nai += dt * (-(ina + ibna + 3 * inak + 3 * inaca) * inverseVcF * CAP);
        Ki += dt * (-(ik1 + ito + ikr + iks - 2 * inak + ipk) * inverseVcF * CAP);
        un[p] -= dt * (ikr + iks + ik1 + ito + ina + ibna + ical + ibca + inak +
                       inaca + ipca + ipk);

        S[S_casr][p] = casr;
        S[S_cass][p] = cass;
        S[S_nai][p] = nai;
        S[S_Ki][p] = Ki;
        S[S_m][p] = m;
        S[S_h][p] = h;
        S[S_j][p] = j;
        S[S_xr1][p] = xr1;
        S[S_xr2][p] = xr2;
        S[S_xs][p] = xs;
        S[S_r][p] = r;
        S[S_s][p] = s;
        S[S_d][p] = d;
        S[S_f][p] = f;
        S[S_f2][p] = f2;
        S[S_fcass][p] = fcass;
        S[S_rr][p] = rr;
        S[S_oo][p] = oo;
        (void)cai;
    }
}

/* ------------------------------------------------------------ Courtemanche */
/* Parameter order (ionic_kernel_2d signature, courtemanche_2d.py:569-577). */
enum {
    C_gna, C_gnab, C_gk1, C_gkr, C_gks, C_gto, C_gcal, C_gcab, C_gkur_coeff,
    C_F, C_T, C_R, C_Vc, C_Vj, C_Vup, C_Vrel, C_ibk, C_cao, C_nao, C_ko,
    C_caupmax, C_kup, C_kmnai, C_kmko, C_kmnancx, C_kmcancx, C_ksatncx,
    C_kmcmdn, C_kmtrpn, C_kmcsqn, C_trpnmax, C_cmdnmax, C_csqnmax,
    C_inacamax, C_inakmax, C_ipcamax, C_krel, C_iupmax, C_kq10, C_NP
};
/* State order (Courtemanche2D.state_vars minus u, courtemanche_2d.py:
 * 118-120): the model's own names. */
enum {
    Q_nai, Q_ki, Q_cai, Q_caup, Q_carel, Q_m, Q_h, Q_j, Q_d, Q_f, Q_oa,
    Q_oi, Q_ua, Q_ui, Q_xr, Q_xs, Q_fca, Q_irel, Q_vrel, Q_urel, Q_wrel,
    Q_NS
};

static inline double gate(double x, double x_inf, double tau_x, double dt)
{
    return x_inf - (x_inf - x) * exp(-dt / tau_x);
}

/* Courtemanche ionic_kernel_2d and its helpers (cpuwave2D/model/
 * courtemanche_2d.py:180-641; 3D courtemanche_3d.py:90-163 per node). */
EXPORT void fwo_ionic_crn(double *un, const double *u, double *const *S,
                          const int64_t *idx, int64_t n_idx, double dt,
                          const double *P)
{
    const double gna = P[C_gna], gnab = P[C_gnab], gk1 = P[C_gk1],
                 gks = P[C_gks], gto = P[C_gto], gcal = P[C_gcal],
                 gcab = P[C_gcab], gkur_coeff = P[C_gkur_coeff], F = P[C_F],
                 T = P[C_T], R = P[C_R], Vj = P[C_Vj], Vup = P[C_Vup],
                 Vrel = P[C_Vrel], ibk = P[C_ibk], cao = P[C_cao],
                 nao = P[C_nao], ko = P[C_ko], caupmax = P[C_caupmax],
                 kup = P[C_kup], kmnai = P[C_kmnai], kmko = P[C_kmko],
                 kmnancx = P[C_kmnancx], kmcancx = P[C_kmcancx],
                 ksatncx = P[C_ksatncx], kmcmdn = P[C_kmcmdn],
                 kmtrpn = P[C_kmtrpn], kmcsqn = P[C_kmcsqn],
                 trpnmax = P[C_trpnmax], cmdnmax = P[C_cmdnmax],
                 csqnmax = P[C_csqnmax], inacamax = P[C_inacamax],
                 inakmax = P[C_inakmax], ipcamax = P[C_ipcamax],
                 krel = P[C_krel], iupmax = P[C_iupmax], kq10 = P[C_kq10];
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_idx; ++t) {
        const int64_t p = idx[t];
        const double uu = u[p];
        double nai = S[Q_nai][p], ki = S[Q_ki][p], cai = S[Q_cai][p],
               caup = S[Q_caup][p], carel = S[Q_carel][p];
        double m = S[Q_m][p], h = S[Q_h][p], j = S[Q_j][p], d = S[Q_d][p],
               f = S[Q_f][p], oa = S[Q_oa][p], oi = S[Q_oi][p],
               ua = S[Q_ua][p], ui = S[Q_ui][p], fca = S[Q_fca][p];
        /* the kernel's `xr` (IKr gate) is the model's xs, its `xs` (IKs
         * gate) the model's xr (argument order, see file header) */
        double g_ikr = S[Q_xs][p], g_iks = S[Q_xr][p];
        double irel = S[Q_irel][p], vrel = S[Q_vrel][p], urel = S[Q_urel][p],
               wrel = S[Q_wrel][p];

        /* calc_equilibrum_potentials (:256-262) */
        const double ena = R * T / F * log(nao / nai);
        const double ek = R * T / F * log(ko / ki);
        const double eca = R * T / (2 * F) * log(cao / cai);
        /* calc_gating_m (:270-282) */
        {
            double am;
            if (uu == -47.13)
                am = 3.2;
            else
                am = 0.32 * (uu + 47.13) / (1 - exp(-0.1 * (uu + 47.13)));
            const double bm = 0.08 * exp(-uu / 11);
            m = gate(m, am / (am + bm), 1 / (am + bm), dt);
        }
        /* calc_gating_h (:285-295) */
        {
            double ah = 0.135 * exp(-(80 + uu) / 6.8);
            double bh = 3.56 * exp(0.079 * uu) + 310000 * exp(0.35 * uu);
            if (uu >= -40) {
                ah = 0;
                bh = 1 / (0.13 * (1 + exp(-(uu + 10.66) / 11.1)));
            }
            h = gate(h, ah / (ah + bh), 1 / (ah + bh), dt);
        }
        /* calc_gating_j (:298-308) */
        {
            double aj = (-127140 * exp(0.2444 * uu) - 3.474e-05 * exp(-0.04391 * uu)) *
                        (uu + 37.78) / (1 + exp(0.311 * (uu + 79.23)));
            double bj = 0.1212 * exp(-0.01052 * uu) / (1 + exp(-0.1378 * (uu + 40.14)));
            if (uu >= -40) {
                aj = 0;
                bj = 0.3 * exp(-2.535e-07 * uu) / (1 + exp(-0.1 * (uu + 32)));
            }
            const double j_inf = aj / (aj + bj);
            const double tau_j = 1 / (aj + bj);
            j = j_inf - (j_inf - j) * exp(-dt / tau_j);
        }
        /* calc_ina (:265-267) */
        const double ina = gna * pow(m, 3) * h * j * (uu - ena);
        /* calc_ik1 (:311-313) */
        const double ik1 = gk1 * (uu - ek) / (1 + exp(0.07 * (uu + 80)));
        /* calc_ito (:316-331) */
        double ito;
        {
            const double ao = 0.65 / (exp(-(uu + 10) / 8.5) + exp(-(uu - 30) / 59.0));
            const double bo = 0.65 / (2.5 + exp((uu + 82) / 17.0));
            const double tau_o = 1 / (kq10 * (ao + bo));
            const double o_inf = 1 / (1 + exp(-(uu + 20.47) / 17.54));
            const double aoi = 1 / (18.53 + exp((uu + 113.7) / 10.95));
            const double boi = 1 / (35.56 + exp(-(uu + 1.26) / 7.44));
            const double tau_oi = 1 / (kq10 * (aoi + boi));
            const double oi_inf = 1 / (1 + exp((uu + 43.1) / 5.3));
            oa = gate(oa, o_inf, tau_o, dt);
            oi = gate(oi, oi_inf, tau_oi, dt);
            ito = gto * pow(oa, 3) * oi * (uu - ek);
        }
        /* calc_ikur (:334-351) */
        double ikur;
        {
            const double gkur = 0.005 + 0.05 / (1 + exp(-(uu - 15) / 13.0));
            const double aua = 0.65 / (exp(-(uu + 10) / 8.5) + exp(-(uu - 30) / 59.0));
            const double bua = 0.65 / (2.5 + exp((uu + 82) / 17.0));
            const double tau_ua = 1 / (kq10 * (aua + bua));
            const double ua_inf = 1 / (1 + exp(-(uu + 30.3) / 9.6));
            const double aui = 1 / (21 + exp(-(uu - 185) / 28.0));
            const double bui = exp((uu - 158) / 16.0);
            const double tau_ui = 1 / (kq10 * (aui + bui));
            const double ui_inf = 1 / (1 + exp((uu - 99.45) / 27.48));
            ua = gate(ua, ua_inf, tau_ua, dt);
            ui = gate(ui, ui_inf, tau_ui, dt);
            ikur = gkur_coeff * gkur * pow(ua, 3) * ui * (uu - ek);
        }
        /* calc_ikr (:354-365), conductance fixed inside the function */
        double ikr;
        {
            const double gkr = 0.0294;
            const double axr = 0.0003 * (uu + 14.1) / (1 - exp(-(uu + 14.1) / 5));
            const double bxr = 7.3898e-05 * (uu - 3.3328) /
                               (exp((uu - 3.3328) / 5.1237) - 1);
            const double tau_xr = 1 / (axr + bxr);
            const double xr_inf = 1 / (1 + exp(-(uu + 14.1) / 6.5));
            g_ikr = gate(g_ikr, xr_inf, tau_xr, dt);
            ikr = gkr * g_ikr * (uu - ek) / (1 + exp((uu + 15) / 22.4));
        }
        /* calc_iks (:368-379) */
        double iks;
        {
            const double axs = 4e-05 * (uu - 19.9) / (1 - exp(-(uu - 19.9) / 17));
            const double bxs = 3.5e-05 * (uu - 19.9) / (exp((uu - 19.9) / 9) - 1);
            const double tau_xs = 1 / (2 * (axs + bxs));
            const double xs_inf = 1 / sqrt(1 + exp(-(uu - 19.9) / 12.7));
            g_iks = gate(g_iks, xs_inf, tau_xs, dt);
            iks = gks * (g_iks * g_iks) * (uu - ek);
        }
        /* calc_ical (:382-396) */
        double ical;
        {
            const double tau_d = (1 - exp(-(uu + 10) / 6.24)) /
                                 (0.035 * (uu + 10) * (1 + exp(-(uu + 10) / 6.24)));
            const double d_inf = 1 / (1 + exp(-(uu + 10) / 8.0));
            const double tau_f = 9 / (0.0197 * exp(-(0.0337 * 0.0337) *
                                                    ((uu + 10) * (uu + 10))) + 0.02);
            const double f_inf = 1 / (1 + exp((uu + 28) / 6.9));
            const double tau_fca = 2;
            const double fca_inf = 1 / (1 + cai / 0.00035);
            d = gate(d, d_inf, tau_d, dt);
            f = gate(f, f_inf, tau_f, dt);
            fca = gate(fca, fca_inf, tau_fca, dt);
            ical = gcal * d * f * fca * (uu - 65);
        }
        /* calc_inak (:399-404) */
        double inak;
        {
            const double s = 1 / 7.0 * (exp(nao / 67.3) - 1);
            const double fnak = 1 / (1 + 0.1245 * exp(-0.1 * (F * uu) / (R * T)) +
                                     0.0365 * s * exp(-(F * uu) / (R * T)));
            inak = inakmax * fnak * (1 / (1 + pow(kmnai / nai, 1.5))) *
                   (ko / (ko + kmko));
        }
        /* calc_inaca (:407-418) */
        double inaca;
        {
            const double gamma = 0.35;
            const double exp_term = exp(gamma * (F * uu) / (R * T));
            const double exp_rev_term = exp((gamma - 1) * (F * uu) / (R * T));
            const double numerator =
                inacamax * (exp_term * pow(nai, 3) * cao -
                            exp_rev_term * pow(nao, 3) * cai);
            const double term1 = pow(kmnancx, 3) + pow(nao, 3);
            const double term2 = kmcancx + cao;
            const double term3 = 1 + ksatncx * exp_rev_term;
            inaca = numerator / (term1 * term2 * term3);
        }
        /* calc_ibca, calc_ibna, calc_ipca (:421-434) */
        const double ibca = gcab * (uu - eca);
        const double ibna = gnab * (uu - ena);
        const double ipca = ipcamax * cai / (cai + 0.0005);
        /* calc_irel (:437-452) */
        {
            const double tau_u = 8;
            const double Fn = 1e-12 * Vrel * irel -
                              5 * 1e-13 / F * (0.5 * ical - 0.2 * inaca);
            const double u_inf = 1 / (1 + exp(-(Fn - 3.4175e-13) / 1.367e-15));
            const double tau_v = 1.91 + 2.09 / (1 + exp(-(Fn - 3.4175e-13) / 1.367e-15));
            const double v_inf = 1 - 1 / (1 + exp(-(Fn - 6.835e-14) / 1.367e-15));
            const double tau_w = 6 * (1 - exp(-(uu - 7.9) / 5.0)) /
                                 ((1 + 0.3 * exp(-(uu - 7.9) / 5.0)) * (uu - 7.9));
            const double w_inf = 1 - 1 / (1 + exp(-(uu - 40) / 17.0));
            urel = gate(urel, u_inf, tau_u, dt);
            vrel = gate(vrel, v_inf, tau_v, dt);
            wrel = gate(wrel, w_inf, tau_w, dt);
            irel = krel * (urel * urel) * vrel * wrel * (carel - cai);
        }
        /* calc_itr, calc_iup, calc_iupleak (:455-469) */
        const double itr = (caup - carel) / 180;
        const double iup = iupmax / (1 + kup / cai);
        const double iupleak = caup / caupmax * iupmax;
        /* calc_caup, calc_nai, calc_ki, calc_cai, calc_carel (:219-253) */
        caup += dt * (iup - iupleak - itr * (Vrel / Vup));
        nai += dt * ((-3 * inak - 3 * inaca - ibna - ina) / (F * Vj));
        ki += dt * ((2 * inak - ik1 - ito - ikur - ikr - iks - ibk) / (F * Vj));
        {
            const double B1 = (2 * inaca - ipca - ical - ibca) / (2 * F * Vj) +
                              (Vup * (iupleak - iup) + irel * Vrel) / Vj;
            const double B2 = 1 + trpnmax * kmtrpn / ((cai + kmtrpn) * (cai + kmtrpn)) +
                              cmdnmax * kmcmdn / ((cai + kmcmdn) * (cai + kmcmdn));
            cai += dt * (B1 / B2);
        }
        carel += dt * ((itr - irel) /
                       (1 + csqnmax * kmcsqn / ((carel + kmcsqn) * (carel + kmcsqn))));
        un[p] -= dt * (ina + ik1 + ito + ikur + ikr + iks + ical + ipca + inak +
                       inaca + ibna + ibca);

        S[Q_nai][p] = nai;
        S[Q_ki][p] = ki;
        S[Q_cai][p] = cai;
        S[Q_caup][p] = caup;
        S[Q_carel][p] = carel;
        S[Q_m][p] = m;
        S[Q_h][p] = h;
        S[Q_j][p] = j;
        S[Q_d][p] = d;
        S[Q_f][p] = f;
        S[Q_oa][p] = oa;
        S[Q_oi][p] = oi;
        S[Q_ua][p] = ua;
        S[Q_ui][p] = ui;
        S[Q_xs][p] = g_ikr;
        S[Q_xr][p] = g_iks;
        S[Q_fca][p] = fca;
        S[Q_irel][p] = irel;
        S[Q_vrel][p] = vrel;
        S[Q_urel][p] = urel;
        S[Q_wrel][p] = wrel;
    }
}

/* ------------------------------------------------------------ Barkley */
/* ionic_kernel_2d (cpuwave2D/model/barkley_2d.py:114-170); P = a, b, eap;
 * S = v. */
EXPORT void fwo_ionic_bk(double *un, const double *u, double *const *S,
                         const int64_t *idx, int64_t n_idx, double dt,
                         const double *P)
{
    const double a = P[0], b = P[1], eap = P[2];
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_idx; ++t) {
        const int64_t p = idx[t];
        const double uu = u[p];
        double v = S[0][p];
        v += dt * (uu - v);
        S[0][p] = v;
        un[p] += dt * (uu * (1 - uu) * (uu - (v + b) / a)) / eap;
    }
}

/* ------------------------------------------------------- Bueno-Orovio */
/* ionic_kernel_2d and calc_* (cpuwave2D/model/bueno_orovio_2d.py:184-460);
 * P in the kernel's parameter order; S = v, w, s. */
EXPORT void fwo_ionic_bo(double *un, const double *u, double *const *S,
                         const int64_t *idx, int64_t n_idx, double dt,
                         const double *P)
{
    const double u_o = P[0], u_u = P[1], theta_v = P[2], theta_w = P[3],
                 theta_v_m = P[4], theta_o = P[5], tau_v1_m = P[6],
                 tau_v2_m = P[7], tau_v_p = P[8], tau_w1_m = P[9],
                 tau_w2_m = P[10], k_w_m = P[11], u_w_m = P[12],
                 tau_w_p = P[13], tau_fi = P[14], tau_o1 = P[15],
                 tau_o2 = P[16], tau_so1 = P[17], tau_so2 = P[18],
                 k_so = P[19], u_so = P[20], tau_s1 = P[21], tau_s2 = P[22],
                 k_s = P[23], u_s = P[24], tau_si = P[25],
                 tau_w_inf = P[26], w_inf_ = P[27];
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_idx; ++t) {
        const int64_t p = idx[t];
        const double uu = u[p];
        double v = S[0][p], w = S[1][p], s = S[2][p];
        const double v_inf = uu < theta_v_m ? 1.0 : 0.0;
        const double tau_v_m = (uu - theta_v_m) < 0 ? tau_v1_m : tau_v2_m;
        const double v_ = (uu - theta_v) < 0 ? (v_inf - v) / tau_v_m
                                             : -v / tau_v_p;
        v += dt * v_;
        const double w_inf = (uu - theta_o) < 0 ? 1 - uu / tau_w_inf : w_inf_;
        const double tau_w_m = tau_w1_m + (tau_w2_m - tau_w1_m) *
                                              (1 + tanh(k_w_m * (uu - u_w_m))) / 2;
        const double w_ = (uu - theta_w) < 0 ? (w_inf - w) / tau_w_m
                                             : -w / tau_w_p;
        w += dt * w_;
        const double tau_s = (uu - theta_w) < 0 ? tau_s1 : tau_s2;
        s += dt * ((1 + tanh(k_s * (uu - u_s))) / 2 - s) / tau_s;
        const double Hv = (uu - theta_v) >= 0 ? 1.0 : 0.0;
        const double J_fi = -v * Hv * (uu - theta_v) * (u_u - uu) / tau_fi;
        const double tau_o = (uu - theta_o) < 0 ? tau_o1 : tau_o2;
        const double tau_so = tau_so1 + (tau_so2 - tau_so1) *
                                            (1 + tanh(k_so * (uu - u_so))) / 2;
        const double Hw = (uu - theta_w) >= 0 ? 1.0 : 0.0;
        const double J_so = (uu - u_o) * (1 - Hw) / tau_o + Hw / tau_so;
        const double J_si = -Hw * w * s / tau_si;
        S[0][p] = v;
        S[1][p] = w;
        S[2][p] = s;
        un[p] += dt * (-J_fi - J_so - J_si);
    }
}

/* ---------------------------------------------------------------- LR91 */
static inline double lr_gate(double var, double dt, double a, double b)
{
    const double tau = 1. / (a + b);
    const double inf = a / (a + b);
    return var + dt * (inf - var) / tau;
}

/* ionic_kernel_2d and calc_* (cpuwave2D/model/luo_rudy91_2d.py); P = gna,
 * gsi, gk, gk1, gkp, gb, ko, ki, nai, nao, cao, R, T, F, PR_NaK; S = m, h,
 * j, d, f, x, cai. */
EXPORT void fwo_ionic_lr91(double *un, const double *u, double *const *S,
                           const int64_t *idx, int64_t n_idx, double dt,
                           const double *P)
{
    const double gna = P[0], gsi = P[1], gk = P[2], gk1 = P[3], gkp = P[4],
                 gb = P[5], ko = P[6], ki = P[7], nai = P[8], nao = P[9],
                 R = P[11], T = P[12], F = P[13], PR_NaK = P[14];
    const double E_Na = (R * T / F) * log(nao / nai);
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_idx; ++t) {
        const int64_t p = idx[t];
        const double uu = u[p];
        double m = S[0][p], h = S[1][p], j = S[2][p], d = S[3][p],
               f = S[4][p], x = S[5][p], cai = S[6][p];
        /* calc_ina */
        double alpha_h = 0, beta_h = 0, beta_J = 0, alpha_J = 0;
        if (uu >= -40.) {
            beta_h = 1. / (0.13 * (1 + exp((uu + 10.66) / -11.1)));
            beta_J = 0.3 * exp(-2.535 * 1e-07 * uu) / (1 + exp(-0.1 * (uu + 32)));
        } else {
            alpha_h = 0.135 * exp((80 + uu) / -6.8);
            beta_h = 3.56 * exp(0.079 * uu) + 3.1 * 1e5 * exp(0.35 * uu);
            beta_J = 0.1212 * exp(-0.01052 * uu) / (1 + exp(-0.1378 * (uu + 40.14)));
            alpha_J = (-1.2714 * 1e5 * exp(0.2444 * uu) -
                       3.474 * 1e-5 * exp(-0.04391 * uu)) *
                      (uu + 37.78) / (1 + exp(0.311 * (uu + 79.23)));
        }
        const double alpha_m = 0.32 * (uu + 47.13) / (1 - exp(-0.1 * (uu + 47.13)));
        const double beta_m = 0.08 * exp(-uu / 11);
        m = lr_gate(m, dt, alpha_m, beta_m);
        h = lr_gate(h, dt, alpha_h, beta_h);
        j = lr_gate(j, dt, alpha_J, beta_J);
        const double ina = gna * m * m * m * h * j * (uu - E_Na);
        /* calc_isk */
        const double E_Si = 7.7 - 13.0287 * log(cai);
        const double isi = gsi * d * f * (uu - E_Si);
        const double alpha_d = 0.095 * exp(-0.01 * (uu - 5)) / (1 + exp(-0.072 * (uu - 5)));
        const double beta_d = 0.07 * exp(-0.017 * (uu + 44)) / (1 + exp(0.05 * (uu + 44)));
        const double alpha_f = 0.012 * exp(-0.008 * (uu + 28)) / (1 + exp(0.15 * (uu + 28)));
        const double beta_f = 0.0065 * exp(-0.02 * (uu + 30)) / (1 + exp(-0.2 * (uu + 30)));
        d = lr_gate(d, dt, alpha_d, beta_d);
        f = lr_gate(f, dt, alpha_f, beta_f);
        cai += dt * (-0.0001 * isi + 0.07 * (0.0001 - cai));
        /* calc_ik */
        const double E_K = (R * T / F) * log((ko + PR_NaK * nao) / (ki + PR_NaK * nai));
        const double G_K = gk * sqrt(ko / 5.4);
        double Xi;
        if (uu > -100)
            Xi = 2.837 * (exp(0.04 * (uu + 77)) - 1) /
                 ((uu + 77) * exp(0.04 * (uu + 35)));
        else
            Xi = 1;
        const double ik = G_K * x * Xi * (uu - E_K);
        const double alpha_x = 0.0005 * exp(0.083 * (uu + 50)) / (1 + exp(0.057 * (uu + 50)));
        const double beta_x = 0.0013 * exp(-0.06 * (uu + 20)) / (1 + exp(-0.04 * (uu + 20)));
        x = lr_gate(x, dt, alpha_x, beta_x);
        const double E_K1 = (R * T / F) * log(ko / ki);
        /* calc_ik1, calc_ikp, calc_ib */
        const double alpha_K1 = 1.02 / (1 + exp(0.2385 * (uu - E_K1 - 59.215)));
        const double beta_K1 = (0.49124 * exp(0.08032 * (uu - E_K1 + 5.476)) +
                                exp(0.06175 * (uu - E_K1 - 594.31))) /
                               (1 + exp(-0.5143 * (uu - E_K1 + 4.753)));
        const double K_1x = alpha_K1 / (alpha_K1 + beta_K1);
        const double G_K1 = gk1 * sqrt(ko / 5.4);
        const double ik1 = G_K1 * K_1x * (uu - E_K1);
        const double K_p = 1. / (1 + exp((7.488 - uu) / 5.98));
        const double ikp = gkp * K_p * (uu - E_K1);
        const double ib = gb * (uu + 59.87);
        const double ik1t = ik1 + ikp + ib;
        un[p] -= dt * (ina + isi + ik1t + ik);
        S[0][p] = m;
        S[1][p] = h;
        S[2][p] = j;
        S[3][p] = d;
        S[4][p] = f;
        S[5][p] = x;
        S[6][p] = cai;
    }
}
