// pnjl_deriv.cu -- implicit derivatives of solved gap-equation states:
// src/pnjl/derivatives/ThermoDerivatives.jl (mass_derivatives :132-173, thermo_derivatives
// :184-249, bulk_viscosity_coefficients :342-465).
//
// The reference differentiates x(theta), theta = (T, mu) with every mu_f moved together, by the
// implicit function theorem (ImplicitDifferentiation.jl) and nested ForwardDiff.  Here, per
// point (one warp), from analytic derivatives:
//   * one FP64 pass with the residual, Hessian and thermo sums (node_pass: the solver's own),
//     assembled into Omega, grad_x Omega, H = Hessian_x Omega, dOmega/dT and rho_f;
//   * one FP64 pass for the theta derivatives: with g = T L(a, b, Phi, Phibar),
//     a = (mu - E)/T, b = -(mu + E)/T, the thermal part is Omega_th = -2 sum_f sum_nodes w g and
//       g_TT = (a^2 L_aa + b^2 L_bb)/T,  g_Tmu = (b L_bb - a L_aa)/T,  g_mumu = (L_aa + L_bb)/T,
//       g_TE = (a L_aa + b L_bb)/T,      g_muE = (L_bb - L_aa)/T,
//       g_TPhi = L_Phi - a L_aPhi - b L_bPhi,  g_muPhi = L_aPhi - L_bPhi   (Phibar alike),
//     with L_a = 3 n+, L_aa = 3 (Phi y + 4 Phibar y^2 + 3 y^3)/f+ - 9 n+^2, L_aPhi = 3 y (1 - 3 n+)/f+,
//     L_aPhibar = 3 y^2 (2 - 3 n+)/f+ (and the antiquark side with Phi <-> Phibar); a factor
//     clamped by the reference's max(f, 1e-16) contributes only its 3a rescaling term;
//   * the Polyakov potential's T derivatives in closed form;
//   * dx/dtheta = -H^-1 d(grad_x Omega)/dtheta (5 x 5 LU, two right-hand sides), then the
//     chain rule for s, n_B, P, eps, M_f and the bulk-viscosity combinations.
// FP64 throughout; not a throughput path (one pass of each kind per point).
#include "pnjl_group.cuh"

namespace pnjl {
namespace {

struct SideD {
    double La, Laa, LaP, LaPb, LP, LPb;  // d/da, d2/da2, d2/dadPhi, d2/dadPhibar, d/dPhi, d/dPhibar
};

// ln f with f = 1 + 3 P y + 3 Pb y^2 + y^3, y = e^a, in the reference's two branches (the
// rescaled one for a > 0) with its max(f, 1e-16) clamp.  P is the Polyakov loop on the y
// term (Phi for quarks, Phibar for antiquarks), Pb the one on the y^2 term.
__device__ __forceinline__ SideD side_derivs(double a, double P, double Pb) {
    double D, N1, N2, r1, r2;
    if (a > 0.0) {
        const double t = exp(-a), t2 = t * t, t3 = t2 * t;
        D = t3 + 3.0 * P * t2 + 3.0 * Pb * t + 1.0;
        N1 = P * t2 + 2.0 * Pb * t + 1.0;
        N2 = P * t2 + 4.0 * Pb * t + 3.0;
        r1 = t2;  // y / y^3
        r2 = t;   // y^2 / y^3
    } else {
        const double y = exp(a), y2 = y * y, y3 = y2 * y;
        D = 1.0 + 3.0 * P * y + 3.0 * Pb * y2 + y3;
        N1 = P * y + 2.0 * Pb * y2 + y3;
        N2 = P * y + 4.0 * Pb * y2 + 3.0 * y3;
        r1 = y;
        r2 = y2;
    }
    SideD s;
    if (D < kPolyakovEps) {  // clamped: only the 3a of the rescaled branch is left
        s.La = a > 0.0 ? 3.0 : 0.0;
        s.Laa = s.LaP = s.LaPb = s.LP = s.LPb = 0.0;
        return s;
    }
    const double iD = 1.0 / D;
    const double n = N1 * iD;
    s.La = 3.0 * n;
    s.Laa = 3.0 * N2 * iD - 9.0 * n * n;
    s.LP = 3.0 * r1 * iD;
    s.LPb = 3.0 * r2 * iD;
    s.LaP = s.LP * (1.0 - 3.0 * n);
    s.LaPb = s.LPb * (2.0 - 3.0 * n);
    return s;
}

// per-flavour theta sums: 0 TT, 1 Tmu, 2 mumu, 3 TM, 4 muM, 5 TPhi, 6 TPhibar, 7 muPhi, 8 muPhibar
constexpr int kDS = 9;

template <int G>
__device__ void deriv_pass(const NodeView &nv, const PointIn &pt, const double *x, const double *M, int gl,
                           unsigned mask, double (&out)[3][kDS]) {
    const int pn = nv.p_num, n = nv.p_num * nv.t_num;
    const double T = pt.T, iT = 1.0 / T, Phi = x[3], Phib = x[4];
    for (int f = 0; f < 3; ++f) {
        double acc[kDS];
#pragma unroll
        for (int k = 0; k < kDS; ++k) acc[k] = 0.0;
        const double mu = pt.mu[f], M2 = M[f] * M[f];
        for (int k = gl; k < n; k += G) {
            const int ip = k % pn, it = k / pn;
            const double w = nv.A[ip] * nv.B[it];
            const double E = sqrt(nv.p2[ip] * (1.0 + pt.xi * nv.c2[it]) + M2);
            const double mE = M[f] / E;
            const double a = (mu - E) * iT, b = -(mu + E) * iT;
            const SideD q = side_derivs(a, Phi, Phib);   // f+ : Phi on y, Phibar on y^2
            const SideD p = side_derivs(b, Phib, Phi);   // f- : Phibar on z, Phi on z^2
            // antiquark side: its "P" slot is Phibar, its "Pb" slot is Phi
            const double LP = q.LP + p.LPb, LPb = q.LPb + p.LP;
            const double LaP = q.LaP, LaPb = q.LaPb, LbP = p.LaPb, LbPb = p.LaP;
            acc[0] += w * (a * a * q.Laa + b * b * p.Laa) * iT;
            acc[1] += w * (b * p.Laa - a * q.Laa) * iT;
            acc[2] += w * (q.Laa + p.Laa) * iT;
            acc[3] += w * (a * q.Laa + b * p.Laa) * iT * mE;
            acc[4] += w * (p.Laa - q.Laa) * iT * mE;
            acc[5] += w * (LP - a * LaP - b * LbP);
            acc[6] += w * (LPb - a * LaPb - b * LbPb);
            acc[7] += w * (LaP - LbP);
            acc[8] += w * (LaPb - LbPb);
        }
#pragma unroll
        for (int k = 0; k < kDS; ++k) out[f][k] = group_sum<G>(acc[k], mask);
    }
}

__device__ __forceinline__ void put(double *dst, int64_t i, double v) {
    if (dst) dst[i] = v;
}

template <int G>
__global__ void __launch_bounds__(kSolveThreads) deriv_kernel(DerivArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const NodeView nv = stage_nodes(a.nodes, smem_raw);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const unsigned mask = group_mask<G>(lane);
    const int64_t groups_per_block = blockDim.x / G;
    const int64_t gid = (int64_t)blockIdx.x * groups_per_block + threadIdx.x / G;
    const int64_t stride = (int64_t)gridDim.x * groups_per_block;
    int64_t evals = 0;
    const DevParams &P = a.P;
    for (int64_t i = gid; i < a.n; i += stride) {
        PointIn pt;
        pt.T = a.T[i];
        pt.mu[0] = a.mu_u[i];
        pt.mu[1] = a.mu_d[i];
        pt.mu[2] = a.mu_s[i];
        pt.xi = a.xi[i];
        double x[5];
        for (int k = 0; k < 5; ++k) x[k] = a.x[5 * i + k];
        double M[3];
        masses(P, x, M);
        PassSums S;
        Eval ev;
        double V, V1[3], V2[3];
        node_pass<double, false, true, true, true, G>(nv, pt, x, M, gl, mask, S, evals);
        vacuum_terms<G>(P, M, gl, mask, lane & ~(G - 1), V, V1, V2);
        assemble<true, true, true>(P, pt, x, M, S, V, V1, V2, ev);
        double D[3][kDS];
        deriv_pass<G>(nv, pt, x, M, gl, mask, D);
        if (gl != 0) continue;
        const double T = pt.T;
        // Polyakov potential: U = -u(T)/2 Phi Phibar + v(T) lg, u = T^4 (a0 + a1 r + a2 r^2),
        // v = T^4 b3 r^3, r = T0/T (Thermodynamics.jl:124-130)
        const double T0 = P.T0, Ph = x[3], Pb = x[4];
        const double du = 4.0 * P.a0 * T * T * T + 3.0 * P.a1 * T0 * T * T + 2.0 * P.a2 * T0 * T0 * T;
        const double d2u = 12.0 * P.a0 * T * T + 6.0 * P.a1 * T0 * T + 2.0 * P.a2 * T0 * T0;
        const double dv = P.b3 * T0 * T0 * T0;
        const double pp = Pb * Ph;
        const double g = 1.0 - 6.0 * pp + 4.0 * (Pb * Pb * Pb + Ph * Ph * Ph) - 3.0 * pp * pp;
        const bool gcl = (g <= 0.0) || (g < kPolyakovEps);
        const double gP = -6.0 * Pb + 12.0 * Ph * Ph - 6.0 * Ph * Pb * Pb;
        const double gPb = -6.0 * Ph + 12.0 * Pb * Pb - 6.0 * Ph * Ph * Pb;
        const double UTT = -0.5 * d2u * pp;
        const double UTP = -0.5 * du * Pb + (gcl ? 0.0 : dv * gP / g);
        const double UTPb = -0.5 * du * Ph + (gcl ? 0.0 : dv * gPb / g);
        // second derivatives of Omega involving theta
        const double G4 = 4.0 * P.G, K2 = 2.0 * P.K;
        const double Jm[3][3] = {{-G4, K2 * x[2], K2 * x[1]}, {K2 * x[2], -G4, K2 * x[0]}, {K2 * x[1], K2 * x[0], -G4}};
        double OTT = UTT, OTM = 0.0, OMM = 0.0, OxT[5], OxM[5];
        for (int f = 0; f < 3; ++f) {
            OTT -= 2.0 * D[f][0];
            OTM -= 2.0 * D[f][1];
            OMM -= 2.0 * D[f][2];
        }
        for (int c = 0; c < 3; ++c) {
            double sT = 0.0, sM = 0.0;
            for (int f = 0; f < 3; ++f) {
                sT += Jm[f][c] * (-2.0 * D[f][3]);
                sM += Jm[f][c] * (-2.0 * D[f][4]);
            }
            OxT[c] = sT;
            OxM[c] = sM;
        }
        OxT[3] = UTP - 2.0 * (D[0][5] + D[1][5] + D[2][5]);
        OxT[4] = UTPb - 2.0 * (D[0][6] + D[1][6] + D[2][6]);
        OxM[3] = -2.0 * (D[0][7] + D[1][7] + D[2][7]);
        OxM[4] = -2.0 * (D[0][8] + D[1][8] + D[2][8]);
        // H = Hessian_x Omega = -J; dx/dtheta = -H^-1 Omega_x,theta
        double H[25], rT[5], rM[5], dxT[5], dxM[5];
        for (int k = 0; k < 25; ++k) H[k] = -ev.J[k];
        for (int k = 0; k < 5; ++k) { rT[k] = -OxT[k]; rM[k] = -OxM[k]; }
        const bool ok = lu_solve5(H, rT, dxT) && lu_solve5(H, rM, dxM);
        const double nanv = qnan();
        if (!ok)
            for (int k = 0; k < 5; ++k) dxT[k] = dxM[k] = nanv;
        // first derivatives: grad_x Omega = -F, Omega_T, Omega_mu = -sum rho_f
        const double OT = ev.dOdT, OM = -(ev.rho[0] + ev.rho[1] + ev.rho[2]);
        double sT = -OTT, sM = -OTM, nT = -OTM, nM = -OMM, PT = -OT, PM = -OM;
        for (int k = 0; k < 5; ++k) {
            sT -= OxT[k] * dxT[k];
            sM -= OxT[k] * dxM[k];
            nT -= OxM[k] * dxT[k];
            nM -= OxM[k] * dxM[k];
            PT += ev.F[k] * dxT[k];  // -grad_x Omega . dx
            PM += ev.F[k] * dxM[k];
        }
        nT /= 3.0;
        nM /= 3.0;
        const double s = -OT, nB = -OM / 3.0, Pv = -ev.omega;
        const double murho = pt.mu[0] * ev.rho[0] + pt.mu[1] * ev.rho[1] + pt.mu[2] * ev.rho[2];
        const double mubar = (pt.mu[0] + pt.mu[1] + pt.mu[2]) / 3.0;
        const double eps = -Pv + murho + T * s;
        const double eT = -PT + mubar * 3.0 * nT + s + T * sT;
        const double eM = -PM + 3.0 * nB + mubar * 3.0 * nM + T * sM;
        const double den_e = eT * nM - eM * nT, den_n = nT * eM - nM * eT;
        const double sMB = sM / 3.0, nMB = nM / 3.0;
        const pnjl_deriv_soa &o = a.out;
        for (int k = 0; k < 5; ++k) {
            if (o.dx_dT) o.dx_dT[5 * i + k] = dxT[k];
            if (o.dx_dmu) o.dx_dmu[5 * i + k] = dxM[k];
        }
        for (int f = 0; f < 3; ++f) {
            double mT = 0.0, mM = 0.0;
            for (int c = 0; c < 3; ++c) { mT += Jm[f][c] * dxT[c]; mM += Jm[f][c] * dxM[c]; }
            if (o.dM_dT) o.dM_dT[3 * i + f] = mT;
            if (o.dM_dmu) o.dM_dmu[3 * i + f] = mM;
        }
        put(o.s, i, s);
        put(o.n_B, i, nB);
        put(o.ds_dT, i, sT);
        put(o.ds_dmu, i, sM);
        put(o.dn_dT, i, nT);
        put(o.dn_dmu, i, nM);
        put(o.pressure, i, Pv);
        put(o.dP_dT, i, PT);
        put(o.dP_dmu, i, PM);
        put(o.energy, i, eps);
        put(o.deps_dT, i, eT);
        put(o.deps_dmu, i, eM);
        put(o.dP_deps_n, i, den_e == 0.0 ? nanv : (PT * nM - PM * nT) / den_e);
        put(o.dP_dn_eps, i, den_n == 0.0 ? nanv : (PT * eM - PM * eT) / den_n);
        put(o.v_n_sq, i, (s * nMB - nB * nT) / (T * (sT * nMB - sMB * nT)));
        put(o.dmuB_dT_sigma, i, -(nB * sT - s * nT) / (nB * sMB - s * nMB));
    }
}

}  // namespace

cudaError_t launch_deriv(const DerivArgs &a, int grid, size_t smem, cudaStream_t s) {
    deriv_kernel<32><<<grid, kSolveThreads, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace pnjl
