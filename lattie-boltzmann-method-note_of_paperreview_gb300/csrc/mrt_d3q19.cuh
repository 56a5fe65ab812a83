// Generated by gen_mrt.py -- do not edit. Sparse D3Q19 MRT relaxation.
// Operator of C/MRT_Process.h:4-179 (f -= Mi S (M f - M feq)) with M, Mi, S of C/MRT_Matrix.h.
#pragma once

// d[q] = F[q] - Feq[q] on entry; on exit F[q] has been relaxed. Rates: s_e (s1), s_eps (s2),
// s_q (s4, s6, s8), s_nu (s9, s11, s13, s14, s15), s_pi (s10, s12), s_m (s16, s17, s18).
template <typename T>
__device__ __forceinline__ void mrt_relax(T (&F)[19], const T (&d)[19], T s_e, T s_eps, T s_q,
                                          T s_nu, T s_pi, T s_m) {
    const T S0 = d[1] + d[2], A0 = d[1] - d[2];
    const T S1 = d[3] + d[4], A1 = d[3] - d[4];
    const T S2 = d[5] + d[6], A2 = d[5] - d[6];
    const T S3 = d[7] + d[10], A3 = d[7] - d[10];
    const T S4 = d[8] + d[9], A4 = d[8] - d[9];
    const T S5 = d[11] + d[14], A5 = d[11] - d[14];
    const T S6 = d[12] + d[13], A6 = d[12] - d[13];
    const T S7 = d[15] + d[18], A7 = d[15] - d[18];
    const T S8 = d[16] + d[17], A8 = d[16] - d[17];
    const T r1 = s_e*T(1.0/2394.0)*(T(-30)*d[0] + T(-11)*(S0 + S1 + S2) + T(8)*(S3 + S4 + S5 + S6 + S7 + S8));
    const T r2 = s_eps*T(1.0/252.0)*(T(12)*d[0] + T(-4)*(S0 + S1 + S2) + (S3 + S4 + S5 + S6 + S7 + S8));
    const T r9 = s_nu*T(1.0/36.0)*(T(-2)*(S7 + S8) + T(2)*S0 - (S1 + S2) + (S3 + S4 + S5 + S6));
    const T r10 = s_pi*T(1.0/72.0)*(T(-4)*S0 + T(-2)*(S7 + S8) + T(2)*(S1 + S2) + (S3 + S4 + S5 + S6));
    const T r11 = s_nu*T(1.0/12.0)*(-(S2 + S5 + S6) + (S1 + S3 + S4));
    const T r12 = s_pi*T(1.0/24.0)*(T(-2)*S1 + T(2)*S2 - (S5 + S6) + (S3 + S4));
    const T r13 = s_nu*T(1.0/4.0)*(-S4 + S3);
    const T r14 = s_nu*T(1.0/4.0)*(-S8 + S7);
    const T r15 = s_nu*T(1.0/4.0)*(-S6 + S5);
    const T r4 = s_q*T(1.0/40.0)*(T(-4)*A0 - (A4 + A6) + (A3 + A5));
    const T r6 = s_q*T(1.0/40.0)*(T(-4)*A1 - A8 + (A3 + A4 + A7));
    const T r8 = s_q*T(1.0/40.0)*(T(-4)*A2 + (A5 + A6 + A7 + A8));
    const T r16 = s_m*T(1.0/8.0)*(-(A4 + A5) + (A3 + A6));
    const T r17 = s_m*T(1.0/8.0)*(-(A3 + A4 + A8) + A7);
    const T r18 = s_m*T(1.0/8.0)*(-(A7 + A8) + (A5 + A6));
    F[0] -= T(-30)*r1 + T(12)*r2;
    { const T ev = T(-11)*r1 + T(-4)*(r2 + r10) + T(2)*r9, od = T(-4)*r4;
      F[1] -= ev + od; F[2] -= ev - od; }
    { const T ev = T(-11)*r1 + T(-4)*r2 + T(-2)*r12 + T(2)*r10 - r9 + r11, od = T(-4)*r6;
      F[3] -= ev + od; F[4] -= ev - od; }
    { const T ev = T(-11)*r1 + T(-4)*r2 + T(2)*(r10 + r12) - (r9 + r11), od = T(-4)*r8;
      F[5] -= ev + od; F[6] -= ev - od; }
    { const T ev = T(8)*r1 + (r2 + r9 + r10 + r11 + r12 + r13), od = -r17 + (r4 + r6 + r16);
      F[7] -= ev + od; F[10] -= ev - od; }
    { const T ev = T(8)*r1 - r13 + (r2 + r9 + r10 + r11 + r12), od = -(r4 + r16 + r17) + r6;
      F[8] -= ev + od; F[9] -= ev - od; }
    { const T ev = T(8)*r1 - (r11 + r12) + (r2 + r9 + r10 + r15), od = -r16 + (r4 + r8 + r18);
      F[11] -= ev + od; F[14] -= ev - od; }
    { const T ev = T(8)*r1 - (r11 + r12 + r15) + (r2 + r9 + r10), od = -r4 + (r8 + r16 + r18);
      F[12] -= ev + od; F[13] -= ev - od; }
    { const T ev = T(8)*r1 + T(-2)*(r9 + r10) + (r2 + r14), od = -r18 + (r6 + r8 + r17);
      F[15] -= ev + od; F[18] -= ev - od; }
    { const T ev = T(8)*r1 + T(-2)*(r9 + r10) - r14 + r2, od = -(r6 + r17 + r18) + r8;
      F[16] -= ev + od; F[17] -= ev - od; }
}

// The same relaxation from d0 = d[0] and the pair sums S[p] = d[a] + d[b] and differences
// A[p] = d[a] - d[b] of the opposite pairs (a, b) = (1,2) (3,4) (5,6) (7,10) (8,9) (11,14) (12,13) (15,18) (16,17).
template <typename T>
__device__ __forceinline__ void mrt_relax_pairs(T (&F)[19], T d0, const T (&S)[9], const T (&A)[9],
                                                T s_e, T s_eps, T s_q, T s_nu, T s_pi, T s_m) {
    const T S0 = S[0], A0 = A[0];
    const T S1 = S[1], A1 = A[1];
    const T S2 = S[2], A2 = A[2];
    const T S3 = S[3], A3 = A[3];
    const T S4 = S[4], A4 = A[4];
    const T S5 = S[5], A5 = A[5];
    const T S6 = S[6], A6 = A[6];
    const T S7 = S[7], A7 = A[7];
    const T S8 = S[8], A8 = A[8];
    const T r1 = s_e*T(1.0/2394.0)*(T(-30)*d0 + T(-11)*(S0 + S1 + S2) + T(8)*(S3 + S4 + S5 + S6 + S7 + S8));
    const T r2 = s_eps*T(1.0/252.0)*(T(12)*d0 + T(-4)*(S0 + S1 + S2) + (S3 + S4 + S5 + S6 + S7 + S8));
    const T r9 = s_nu*T(1.0/36.0)*(T(-2)*(S7 + S8) + T(2)*S0 - (S1 + S2) + (S3 + S4 + S5 + S6));
    const T r10 = s_pi*T(1.0/72.0)*(T(-4)*S0 + T(-2)*(S7 + S8) + T(2)*(S1 + S2) + (S3 + S4 + S5 + S6));
    const T r11 = s_nu*T(1.0/12.0)*(-(S2 + S5 + S6) + (S1 + S3 + S4));
    const T r12 = s_pi*T(1.0/24.0)*(T(-2)*S1 + T(2)*S2 - (S5 + S6) + (S3 + S4));
    const T r13 = s_nu*T(1.0/4.0)*(-S4 + S3);
    const T r14 = s_nu*T(1.0/4.0)*(-S8 + S7);
    const T r15 = s_nu*T(1.0/4.0)*(-S6 + S5);
    const T r4 = s_q*T(1.0/40.0)*(T(-4)*A0 - (A4 + A6) + (A3 + A5));
    const T r6 = s_q*T(1.0/40.0)*(T(-4)*A1 - A8 + (A3 + A4 + A7));
    const T r8 = s_q*T(1.0/40.0)*(T(-4)*A2 + (A5 + A6 + A7 + A8));
    const T r16 = s_m*T(1.0/8.0)*(-(A4 + A5) + (A3 + A6));
    const T r17 = s_m*T(1.0/8.0)*(-(A3 + A4 + A8) + A7);
    const T r18 = s_m*T(1.0/8.0)*(-(A7 + A8) + (A5 + A6));
    F[0] -= T(-30)*r1 + T(12)*r2;
    { const T ev = T(-11)*r1 + T(-4)*(r2 + r10) + T(2)*r9, od = T(-4)*r4;
      F[1] -= ev + od; F[2] -= ev - od; }
    { const T ev = T(-11)*r1 + T(-4)*r2 + T(-2)*r12 + T(2)*r10 - r9 + r11, od = T(-4)*r6;
      F[3] -= ev + od; F[4] -= ev - od; }
    { const T ev = T(-11)*r1 + T(-4)*r2 + T(2)*(r10 + r12) - (r9 + r11), od = T(-4)*r8;
      F[5] -= ev + od; F[6] -= ev - od; }
    { const T ev = T(8)*r1 + (r2 + r9 + r10 + r11 + r12 + r13), od = -r17 + (r4 + r6 + r16);
      F[7] -= ev + od; F[10] -= ev - od; }
    { const T ev = T(8)*r1 - r13 + (r2 + r9 + r10 + r11 + r12), od = -(r4 + r16 + r17) + r6;
      F[8] -= ev + od; F[9] -= ev - od; }
    { const T ev = T(8)*r1 - (r11 + r12) + (r2 + r9 + r10 + r15), od = -r16 + (r4 + r8 + r18);
      F[11] -= ev + od; F[14] -= ev - od; }
    { const T ev = T(8)*r1 - (r11 + r12 + r15) + (r2 + r9 + r10), od = -r4 + (r8 + r16 + r18);
      F[12] -= ev + od; F[13] -= ev - od; }
    { const T ev = T(8)*r1 + T(-2)*(r9 + r10) + (r2 + r14), od = -r18 + (r6 + r8 + r17);
      F[15] -= ev + od; F[18] -= ev - od; }
    { const T ev = T(8)*r1 + T(-2)*(r9 + r10) - r14 + r2, od = -(r6 + r17 + r18) + r8;
      F[16] -= ev + od; F[17] -= ev - od; }
}

// Non-equilibrium momentum flux Pi_ab = sum_q e_qa e_qb d_q, returned as Q = Pi:Pi.
template <typename T>
__device__ __forceinline__ T pi_neq_norm2(const T (&d)[19]) {
    const T S0 = d[1] + d[2];
    const T S1 = d[3] + d[4];
    const T S2 = d[5] + d[6];
    const T S3 = d[7] + d[10];
    const T S4 = d[8] + d[9];
    const T S5 = d[11] + d[14];
    const T S6 = d[12] + d[13];
    const T S7 = d[15] + d[18];
    const T S8 = d[16] + d[17];
    const T pxx = (S0 + S3 + S4 + S5 + S6);
    const T pyy = (S1 + S3 + S4 + S7 + S8);
    const T pzz = (S2 + S5 + S6 + S7 + S8);
    const T pxy = -S4 + S3;
    const T pyz = -S8 + S7;
    const T pxz = -S6 + S5;
    return pxx*pxx + pyy*pyy + pzz*pzz + T(2)*(pxy*pxy + pyz*pyz + pxz*pxz);
}

// The same from the pair sums S[p] = d[a] + d[b].
template <typename T>
__device__ __forceinline__ T pi_neq_norm2_pairs(const T (&S)[9]) {
    const T pxx = (S[0] + S[3] + S[4] + S[5] + S[6]);
    const T pyy = (S[1] + S[3] + S[4] + S[7] + S[8]);
    const T pzz = (S[2] + S[5] + S[6] + S[7] + S[8]);
    const T pxy = -S[4] + S[3];
    const T pyz = -S[8] + S[7];
    const T pxz = -S[6] + S[5];
    return pxx*pxx + pyy*pyy + pzz*pzz + T(2)*(pxy*pxy + pyz*pyz + pxz*pxz);
}
