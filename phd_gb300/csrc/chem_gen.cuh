// Generated by phd_gb300/mechgen.py from phd_gb300/data/h2_sandiego12.inp -- do not edit.
// The constant-volume reactor right-hand side of this mechanism (9 species,
// 12 reactions) as straight-line code: the expressions and operation order of
// fun_tpart / fun_cpart in chem.cu with the mechanism's tables as literals.
#pragma once

namespace chem_gen {

constexpr int KK = 9;

// temperature terms of one right-hand side; the finite-difference Jacobian's
// species columns reuse them (rc_drive)
struct FunT {
  double T;
  double rut;
  double cvk[9], h[9];
  double kf[12];
  double kr[6];   // reactions 0, 1, 2, 5, 7, 8
  double klow[2];   // reactions 3, 11
  double fclog[2];   // reactions 3, 11
};

HD __forceinline__ void tpart(double T, FunT& t) {
  const double Tinv = 1.0 / T;
  const double alogt = log(T);
  const double T2 = T * T, T3 = T * T2, T4 = T2 * T2;
  t.T = T;
  t.rut = T * 0x1.3d2c630000000p+26;
  {   // species 0
    const bool hi = T > 0x1.f400000000000p+9;
    const double a0 = hi ? 0x1.40000015798eep+1 : 0x1.4000000000000p+1;
    const double a1 = hi ? (-0x1.961a6ec6a1e45p-36) : 0x1.8d112bff6d580p-41;
    const double a2 = hi ? 0x1.230b4c341c642p-46 : (-0x1.1fa470055807fp-49);
    const double a3 = hi ? (-0x1.5d647fbe2e672p-58) : 0x1.538a620b2373fp-59;
    const double a4 = hi ? 0x1.2d244e9510ba2p-71 : (-0x1.1863cffe0b329p-70);
    const double a5 = hi ? 0x1.8e06a3bcd35a8p+14 : 0x1.8e06a3bcd35a8p+14;
    const double cps = a0 + T * a1 + T2 * a2 + T3 * a3 + T4 * a4;
    t.cvk[0] = 0x1.3aaa5ed0194dcp+26 * (cps - 1.0);
    const double hs = a0 + (0.5 * T) * a1 + (T2 * (1.0 / 3.0)) * a2 + (0.25 * T3) * a3 + (0.2 * T4) * a4;
    t.h[0] = t.rut * (hs + a5 * Tinv) * 0x1.fbf39e8ab06bdp-1;
  }
  {   // species 1
    const bool hi = T > 0x1.f400000000000p+9;
    const double a0 = hi ? 0x1.ab2bf6fecf7e5p+1 : 0x1.2c130ac9b2911p+1;
    const double a1 = hi ? (-0x1.9e6b00cea2ba4p-15) : 0x1.058175d02a941p-7;
    const double a2 = hi ? 0x1.0c24d11e93b22p-21 : (-0x1.46ca05831775cp-16);
    const double a3 = hi ? (-0x1.8adee4a4b6baep-33) : 0x1.5a4c582f87e3dp-26;
    const double a4 = hi ? 0x1.68bf7de4136dcp-46 : (-0x1.03862939e564dp-37);
    const double a5 = hi ? (-0x1.db14578e5c4ebp+9) : (-0x1.caf7b3bfb58d1p+9);
    const double cps = a0 + T * a1 + T2 * a2 + T3 * a3 + T4 * a4;
    t.cvk[1] = 0x1.3aaa5ed0194dcp+25 * (cps - 1.0);
    const double hs = a0 + (0.5 * T) * a1 + (T2 * (1.0 / 3.0)) * a2 + (0.25 * T3) * a3 + (0.2 * T4) * a4;
    t.h[1] = t.rut * (hs + a5 * Tinv) * 0x1.fbf39e8ab06bdp-2;
  }
  {   // species 2
    const bool hi = T > 0x1.f400000000000p+9;
    const double a0 = hi ? 0x1.48e2c7b5e1a3dp+1 : 0x1.9589c6bdbf12dp+1;
    const double a1 = hi ? (-0x1.689a006cdb509p-14) : (-0x1.add3ae5787a18p-9);
    const double a2 = hi ? 0x1.6855a2fbdda5cp-25 : 0x1.bdcef845b6ae0p-18;
    const double a3 = hi ? (-0x1.607823c010ceap-37) : (-0x1.a51e14d5c0503p-28);
    const double a4 = hi ? 0x1.620b4436bd152p-50 : 0x1.2954967e1b470p-39;
    const double a5 = hi ? 0x1.c88650ff97247p+14 : 0x1.c709096bb98c8p+14;
    const double cps = a0 + T * a1 + T2 * a2 + T3 * a3 + T4 * a4;
    t.cvk[2] = 0x1.3d2f6e558a183p+22 * (cps - 1.0);
    const double hs = a0 + (0.5 * T) * a1 + (T2 * (1.0 / 3.0)) * a2 + (0.25 * T3) * a3 + (0.2 * T4) * a4;
    t.h[2] = t.rut * (hs + a5 * Tinv) * 0x1.000275060987dp-4;
  }
  {   // species 3
    const bool hi = T > 0x1.f400000000000p+9;
    const double a0 = hi ? 0x1.a42a332f575b8p+1 : 0x1.e42787ae5fa45p+1;
    const double a1 = hi ? 0x1.84c851ecf574dp-10 : (-0x1.88c9b66c8c0dfp-9);
    const double a2 = hi ? (-0x1.96ee255022a3dp-21) : 0x1.4a6bae1fdae75p-17;
    const double a3 = hi ? 0x1.cca1706e20348p-33 : (-0x1.4ca5927ada53cp-27);
    const double a4 = hi ? (-0x1.8667712a69c18p-46) : 0x1.c883a18b02bcdp-39;
    const double a5 = hi ? (-0x1.101d4b48d3ae7p+10) : (-0x1.09fc63497b741p+10);
    const double cps = a0 + T * a1 + T2 * a2 + T3 * a3 + T4 * a4;
    t.cvk[3] = 0x1.3d2f6e558a183p+21 * (cps - 1.0);
    const double hs = a0 + (0.5 * T) * a1 + (T2 * (1.0 / 3.0)) * a2 + (0.25 * T3) * a3 + (0.2 * T4) * a4;
    t.h[3] = t.rut * (hs + a5 * Tinv) * 0x1.000275060987dp-5;
  }
  {   // species 4
    const bool hi = T > 0x1.f400000000000p+9;
    const double a0 = hi ? 0x1.8be3be406d029p+1 : 0x1.fefa5c927d1abp+1;
    const double a1 = hi ? 0x1.1f88fd8e1440ep-11 : (-0x1.3abed86e71c7dp-9);
    const double a2 = hi ? 0x1.0faafc0d73234p-23 : 0x1.35e793e99fbcdp-18;
    const double a3 = hi ? (-0x1.82ca91827ab6dp-34) : (-0x1.0ab59e9e67441p-28);
    const double a4 = hi ? 0x1.a705cd746f5f8p-47 : 0x1.7ff6d2c211dd3p-40;
    const double a5 = hi ? 0x1.e2550624dd2f2p+11 : 0x1.c3e293f290abbp+11;
    const double cps = a0 + T * a1 + T2 * a2 + T3 * a3 + T4 * a4;
    t.cvk[4] = 0x1.2a63031c056b1p+22 * (cps - 1.0);
    const double hs = a0 + (0.5 * T) * a1 + (T2 * (1.0 / 3.0)) * a2 + (0.25 * T3) * a3 + (0.2 * T4) * a4;
    t.h[4] = t.rut * (hs + a5 * Tinv) * 0x1.e1ac6c774b6a9p-5;
  }
  {   // species 5
    const bool hi = T > 0x1.f400000000000p+9;
    const double a0 = hi ? 0x1.8459ddac6e07ap+1 : 0x1.0cb686e536fbfp+2;
    const double a1 = hi ? 0x1.1d553f9364039p-9 : (-0x1.0aeb63b84c925p-9);
    const double a2 = hi ? (-0x1.6057d217698d4p-23) : 0x1.b593a7c039b70p-18;
    const double a3 = hi ? (-0x1.aacb906a5f7ccp-34) : (-0x1.7921667072d59p-28);
    const double a4 = hi ? 0x1.2f01042cd6ffep-46 : 0x1.f2c47bce627b1p-40;
    const double a5 = hi ? (-0x1.d4d1303afb7e9p+14) : (-0x1.d956e8240b780p+14);
    const double cps = a0 + T * a1 + T2 * a2 + T3 * a3 + T4 * a4;
    t.cvk[5] = 0x1.19b11bf5ba9e9p+22 * (cps - 1.0);
    const double hs = a0 + (0.5 * T) * a1 + (T2 * (1.0 / 3.0)) * a2 + (0.25 * T3) * a3 + (0.2 * T4) * a4;
    t.h[5] = t.rut * (hs + a5 * Tinv) * 0x1.c6b93cc1512cbp-5;
  }
  {   // species 6
    const bool hi = T > 0x1.f400000000000p+9;
    const double a0 = hi ? 0x1.0119fbbf289f6p+2 : 0x1.1350a899bcaa1p+2;
    const double a1 = hi ? 0x1.2593e46a1f9dfp-9 : (-0x1.373d054674594p-8);
    const double a2 = hi ? (-0x1.5431502070c84p-21) : 0x1.62fa28e3a8ea6p-16;
    const double a3 = hi ? 0x1.f675fa32f618cp-34 : (-0x1.a110b0905e0fcp-26);
    const double a4 = hi ? (-0x1.84c80e71ea191p-47) : 0x1.46f1288fc5c1cp-37;
    const double a5 = hi ? 0x1.bf6d462c343b7p+6 : 0x1.26cedbb59ddc2p+8;
    const double cps = a0 + T * a1 + T2 * a2 + T3 * a3 + T4 * a4;
    t.cvk[6] = 0x1.337fbd7576e8bp+21 * (cps - 1.0);
    const double hs = a0 + (0.5 * T) * a1 + (T2 * (1.0 / 3.0)) * a2 + (0.25 * T3) * a3 + (0.2 * T4) * a4;
    t.h[6] = t.rut * (hs + a5 * Tinv) * 0x1.f0620d016f133p-6;
  }
  {   // species 7
    const bool hi = T > 0x1.f400000000000p+9;
    const double a0 = hi ? 0x1.0a8f681d1fcb7p+2 : 0x1.11abd48f63e0ap+2;
    const double a1 = hi ? 0x1.41abe4bc5704bp-8 : (-0x1.1c98643a78c6ap-11);
    const double a2 = hi ? (-0x1.fe66ae3495cc5p-20) : 0x1.18be22e62f026p-16;
    const double a3 = hi ? 0x1.981f91177d524p-32 : (-0x1.72b101d35ae59p-26);
    const double a4 = hi ? (-0x1.0353229ef325dp-45) : 0x1.2f72fba30b7c2p-37;
    const double a5 = hi ? (-0x1.1717269ad42c4p+14) : (-0x1.149a541205bc0p+14);
    const double cps = a0 + T * a1 + T2 * a2 + T3 * a3 + T4 * a4;
    t.cvk[7] = 0x1.2a63031c056b1p+21 * (cps - 1.0);
    const double hs = a0 + (0.5 * T) * a1 + (T2 * (1.0 / 3.0)) * a2 + (0.25 * T3) * a3 + (0.2 * T4) * a4;
    t.h[7] = t.rut * (hs + a5 * Tinv) * 0x1.e1ac6c774b6a9p-6;
  }
  {   // species 8
    const bool hi = T > 0x1.f400000000000p+9;
    const double a0 = hi ? 0x1.769c23b7952d2p+1 : 0x1.a63b0c4588a05p+1;
    const double a1 = hi ? 0x1.86106ec5d7fc6p-10 : 0x1.712969da04050p-10;
    const double a2 = hi ? (-0x1.3132bf1b89c39p-21) : (-0x1.09f7a2b098bd4p-18);
    const double a3 = hi ? 0x1.bc128a9b8a724p-34 : 0x1.83ae94da0fe59p-28;
    const double a4 = hi ? (-0x1.e6a15668d1fd9p-48) : (-0x1.581526048e0d6p-39);
    const double a5 = hi ? (-0x1.cd661b089a027p+9) : (-0x1.fe732fec56d5dp+9);
    const double cps = a0 + T * a1 + T2 * a2 + T3 * a3 + T4 * a4;
    t.cvk[8] = 0x1.6a4f7c37c9782p+21 * (cps - 1.0);
    const double hs = a0 + (0.5 * T) * a1 + (T2 * (1.0 / 3.0)) * a2 + (0.25 * T3) * a3 + (0.2 * T4) * a4;
    t.h[8] = t.rut * (hs + a5 * Tinv) * 0x1.246e76057aa8cp-5;
  }
  t.kf[0] = 0x1.f438daa060000p+54 * exp((-0x1.6666666666666p-1) * alogt - 0x1.0c6f4493ef159p+13 * Tinv);
  t.kr[0] = 0x1.001d1bf800000p+46 * exp((-0x1.0a3d70a3d70a4p-2) * alogt - 0x1.1fd705d6afec6p+6 * Tinv);
  t.kf[1] = 0x1.8b50000000000p+15 * exp(0x1.55c28f5c28f5cp+1 * alogt - 0x1.8bb78dad5b973p+11 * Tinv);
  t.kr[1] = 0x1.d970000000000p+14 * exp(0x1.50a3d70a3d70ap+1 * alogt - 0x1.3072327bb03a1p+11 * Tinv);
  t.kf[2] = 0x1.16f3220000000p+30 * exp(0x1.4cccccccccccdp+0 * alogt - 0x1.c94c533be761cp+10 * Tinv);
  t.kr[2] = 0x1.7d78400000000p+33 * exp(0x1.30a3d70a3d70ap+0 * alogt - 0x1.2611369490098p+13 * Tinv);
  t.kf[3] = 0x1.0eaa664900000p+42 * exp(0x1.c28f5c28f5c29p-2 * alogt - 0.0 * Tinv);
  t.klow[0] = 0x1.8efc84ad0c7b0p+65 * exp((-0x1.6666666666666p+0) * alogt - 0.0 * Tinv);
  {
    const double ta = 0x1.0000000000000p-1;
    double fcent = (1.0 - ta) * exp(-T * 0x1.93e5939a08ce9p+99) + ta * exp(-T * 0x1.4484bfeebc29fp-100);
    t.fclog[0] = log(fmax(fcent, 1.0e-300)) * 0.4342944819032518277;
  }
  t.kf[4] = 0x1.0191a36680000p+46 * exp(0.0 * alogt - 0x1.27e432c1d6dbcp+7 * Tinv);
  t.kf[5] = 0x1.e31fa34e00000p+43 * exp(0.0 * alogt - 0x1.9da4e3b0f0481p+8 * Tinv);
  t.kr[3] = 0x1.39283f4a00000p+41 * exp(0x1.70a3d70a3d70ap-2 * alogt - 0x1.b3c1120ab0336p+14 * Tinv);
  t.kf[6] = 0x1.a48ce3be80000p+44 * exp(0.0 * alogt - (-0x1.f4328690d2d50p+7) * Tinv);
  t.kf[7] = 0x1.0f0cf064dd592p+75 * exp((-0x1.0000000000000p+1) * alogt - 0.0 * Tinv);
  t.kr[4] = 0x1.5cfa424ea9c92p+76 * exp((-0x1.c000000000000p+0) * alogt - 0x1.d22edd4d65d8ep+15 * Tinv);
  t.kf[8] = 0x1.20a871cc00200p+60 * exp((-0x1.0000000000000p+0) * alogt - 0.0 * Tinv);
  t.kr[5] = 0x1.0e0198eaee000p+58 * exp((-0x1.4cccccccccccdp-1) * alogt - 0x1.96e5d98de8289p+15 * Tinv);
  t.kf[9] = 0x1.5f93037c00000p+41 * exp(0.0 * alogt - 0x1.5dbc4f266b3c5p+9 * Tinv);
  t.kf[10] = 0x1.2dbf9ea000000p+37 * exp(0x1.3851eb851eb85p-1 * alogt - 0x1.784fcc6a9ac05p+13 * Tinv);
  t.kf[11] = 0x1.6b99192fbb3c0p+64 * exp((-0x1.63d70a3d70a3dp+0) * alogt - 0x1.93845131294f1p+14 * Tinv);
  t.klow[1] = 0x1.592a7a2071df8p+79 * exp((-0x1.e666666666666p+0) * alogt - 0x1.8626719ec5abbp+14 * Tinv);
  {
    const double ta = 0x1.7851eb851eb85p-1;
    double fcent = (1.0 - ta) * exp(-T * 0x1.5c9882b931057p-7) + ta * exp(-T * 0x1.2a91c92f3c105p-11);
    fcent = fcent + exp(-0x1.43e0000000000p+12 * Tinv);
    t.fclog[1] = log(fmax(fcent, 1.0e-300)) * 0.4342944819032518277;
  }
}

HD __forceinline__ void cpart(double rho, const double* z, const FunT& t, double* zp) {
  const double* Y = z + 1;
  double cv = 0.0, ctot = 0.0;
  cv = cv + Y[0] * t.cvk[0];
  const double C0 = rho * Y[0] * 0x1.fbf39e8ab06bdp-1;
  ctot = ctot + C0;
  cv = cv + Y[1] * t.cvk[1];
  const double C1 = rho * Y[1] * 0x1.fbf39e8ab06bdp-2;
  ctot = ctot + C1;
  cv = cv + Y[2] * t.cvk[2];
  const double C2 = rho * Y[2] * 0x1.000275060987dp-4;
  ctot = ctot + C2;
  cv = cv + Y[3] * t.cvk[3];
  const double C3 = rho * Y[3] * 0x1.000275060987dp-5;
  ctot = ctot + C3;
  cv = cv + Y[4] * t.cvk[4];
  const double C4 = rho * Y[4] * 0x1.e1ac6c774b6a9p-5;
  ctot = ctot + C4;
  cv = cv + Y[5] * t.cvk[5];
  const double C5 = rho * Y[5] * 0x1.c6b93cc1512cbp-5;
  ctot = ctot + C5;
  cv = cv + Y[6] * t.cvk[6];
  const double C6 = rho * Y[6] * 0x1.f0620d016f133p-6;
  ctot = ctot + C6;
  cv = cv + Y[7] * t.cvk[7];
  const double C7 = rho * Y[7] * 0x1.e1ac6c774b6a9p-6;
  ctot = ctot + C7;
  cv = cv + Y[8] * t.cvk[8];
  const double C8 = rho * Y[8] * 0x1.246e76057aa8cp-5;
  ctot = ctot + C8;
  double rop0;
  {   // reaction 0
    double rkft = t.kf[0];
    double rkrt = t.kr[0];
    double rkf = rkft * C0;
    double rkr = rkrt * C2;
    rkf = rkf * C3;
    rkr = rkr * C4;
    rop0 = rkf - rkr;
  }
  double rop1;
  {   // reaction 1
    double rkft = t.kf[1];
    double rkrt = t.kr[1];
    double rkf = rkft * C1;
    double rkr = rkrt * C0;
    rkf = rkf * C2;
    rkr = rkr * C4;
    rop1 = rkf - rkr;
  }
  double rop2;
  {   // reaction 2
    double rkft = t.kf[2];
    double rkrt = t.kr[2];
    double rkf = rkft * C1;
    double rkr = rkrt * C0;
    rkf = rkf * C4;
    rkr = rkr * C5;
    rop2 = rkf - rkr;
  }
  double rop3;
  {   // reaction 3
    double rkft = t.kf[3];
    double ctb = ctot;
    ctb = ctb + 0x1.8000000000000p+0 * C1;
    ctb = ctb + 0x1.e000000000000p+3 * C5;
    const double pr = t.klow[0] * ctb / rkft;
    double pcor = pr / (1.0 + pr);
    {
      const double prlog = log(fmax(pr, 1.0e-300)) * 0.4342944819032518277;
      const double fclog = t.fclog[0];
      const double xn = 0.75 - 1.27 * fclog;
      const double cprlog = prlog - (0.4 + 0.67 * fclog);
      const double q = cprlog / (xn - 0.14 * cprlog);
      const double flog = fclog / (1.0 + q * q);
      pcor = exp(flog * 2.302585092994045684) * pcor;
    }
    rkft = rkft * pcor;
    double rkf = rkft * C0;
    rkf = rkf * C3;
    rop3 = rkf;
  }
  double rop4;
  {   // reaction 4
    double rkft = t.kf[4];
    double rkf = rkft * C0;
    rkf = rkf * C6;
    rop4 = rkf;
  }
  double rop5;
  {   // reaction 5
    double rkft = t.kf[5];
    double rkrt = t.kr[3];
    double rkf = rkft * C0;
    double rkr = rkrt * C1;
    rkf = rkf * C6;
    rkr = rkr * C3;
    rop5 = rkf - rkr;
  }
  double rop6;
  {   // reaction 6
    double rkft = t.kf[6];
    double rkf = rkft * C4;
    rkf = rkf * C6;
    rop6 = rkf;
  }
  double rop7;
  {   // reaction 7
    double rkft = t.kf[7];
    double rkrt = t.kr[4];
    double ctb = ctot;
    ctb = ctb + 0x1.8000000000000p+0 * C1;
    ctb = ctb + 0x1.6000000000000p+3 * C5;
    rkft = rkft * ctb;
    rkrt = rkrt * ctb;
    double rkf = rkft * C0;
    double rkr = rkrt * C5;
    rkf = rkf * C4;
    rop7 = rkf - rkr;
  }
  double rop8;
  {   // reaction 8
    double rkft = t.kf[8];
    double rkrt = t.kr[5];
    double ctb = ctot;
    ctb = ctb + 0x1.8000000000000p+0 * C1;
    ctb = ctb + 0x1.6000000000000p+3 * C5;
    rkft = rkft * ctb;
    rkrt = rkrt * ctb;
    double rkf = rkft * (C0 * C0);
    double rkr = rkrt * C1;
    rop8 = rkf - rkr;
  }
  double rop9;
  {   // reaction 9
    double rkft = t.kf[9];
    double rkf = rkft * (C6 * C6);
    rop9 = rkf;
  }
  double rop10;
  {   // reaction 10
    double rkft = t.kf[10];
    double rkf = rkft * C1;
    rkf = rkf * C6;
    rop10 = rkf;
  }
  double rop11;
  {   // reaction 11
    double rkft = t.kf[11];
    double ctb = ctot;
    ctb = ctb + 0x1.8000000000000p+0 * C1;
    ctb = ctb + 0x1.4000000000000p+2 * C5;
    const double pr = t.klow[1] * ctb / rkft;
    double pcor = pr / (1.0 + pr);
    {
      const double prlog = log(fmax(pr, 1.0e-300)) * 0.4342944819032518277;
      const double fclog = t.fclog[1];
      const double xn = 0.75 - 1.27 * fclog;
      const double cprlog = prlog - (0.4 + 0.67 * fclog);
      const double q = cprlog / (xn - 0.14 * cprlog);
      const double flog = fclog / (1.0 + q * q);
      pcor = exp(flog * 2.302585092994045684) * pcor;
    }
    rkft = rkft * pcor;
    double rkf = rkft * C7;
    rop11 = rkf;
  }
  const double wdot0 = (((((((((0.0 + rop0 * (-0x1.0000000000000p+0)) + rop3 * (-0x1.0000000000000p+0)) + rop4 * (-0x1.0000000000000p+0)) + rop5 * (-0x1.0000000000000p+0)) + rop7 * (-0x1.0000000000000p+0)) + rop8 * (-0x1.0000000000000p+1)) + rop1 * 0x1.0000000000000p+0) + rop2 * 0x1.0000000000000p+0) + rop10 * 0x1.0000000000000p+0);
  const double wdot1 = (((((0.0 + rop1 * (-0x1.0000000000000p+0)) + rop2 * (-0x1.0000000000000p+0)) + rop10 * (-0x1.0000000000000p+0)) + rop5 * 0x1.0000000000000p+0) + rop8 * 0x1.0000000000000p+0);
  const double wdot2 = ((0.0 + rop1 * (-0x1.0000000000000p+0)) + rop0 * 0x1.0000000000000p+0);
  const double wdot3 = (((((0.0 + rop0 * (-0x1.0000000000000p+0)) + rop3 * (-0x1.0000000000000p+0)) + rop6 * 0x1.0000000000000p+0) + rop9 * 0x1.0000000000000p+0) + rop5 * 0x1.0000000000000p+0);
  const double wdot4 = (((((((0.0 + rop6 * (-0x1.0000000000000p+0)) + rop2 * (-0x1.0000000000000p+0)) + rop7 * (-0x1.0000000000000p+0)) + rop4 * 0x1.0000000000000p+1) + rop11 * 0x1.0000000000000p+1) + rop0 * 0x1.0000000000000p+0) + rop1 * 0x1.0000000000000p+0);
  const double wdot5 = (((0.0 + rop7 * 0x1.0000000000000p+0) + rop2 * 0x1.0000000000000p+0) + rop6 * 0x1.0000000000000p+0);
  const double wdot6 = ((((((0.0 + rop9 * (-0x1.0000000000000p+1)) + rop4 * (-0x1.0000000000000p+0)) + rop5 * (-0x1.0000000000000p+0)) + rop6 * (-0x1.0000000000000p+0)) + rop10 * (-0x1.0000000000000p+0)) + rop3 * 0x1.0000000000000p+0);
  const double wdot7 = (((0.0 + rop11 * (-0x1.0000000000000p+0)) + rop9 * 0x1.0000000000000p+0) + rop10 * 0x1.0000000000000p+0);
  const double wdot8 = 0.0;
  const double rho_i = 1.0 / rho;
  double sum = 0.0;
  zp[1] = wdot0 * 0x1.020a520000000p+0 * rho_i;
  sum = sum + t.h[0] * wdot0 * 0x1.020a520000000p+0 + (-t.rut) * wdot0;
  zp[2] = wdot1 * 0x1.020a520000000p+1 * rho_i;
  sum = sum + t.h[1] * wdot1 * 0x1.020a520000000p+1 + (-t.rut) * wdot1;
  zp[3] = wdot2 * 0x1.fffb160000000p+3 * rho_i;
  sum = sum + t.h[2] * wdot2 * 0x1.fffb160000000p+3 + (-t.rut) * wdot2;
  zp[4] = wdot3 * 0x1.fffb160000000p+4 * rho_i;
  sum = sum + t.h[3] * wdot3 * 0x1.fffb160000000p+4 + (-t.rut) * wdot3;
  zp[5] = wdot4 * 0x1.101e302000000p+4 * rho_i;
  sum = sum + t.h[4] * wdot4 * 0x1.101e302000000p+4 + (-t.rut) * wdot4;
  zp[6] = wdot5 * 0x1.203ed54000000p+4 * rho_i;
  sum = sum + t.h[5] * wdot5 * 0x1.203ed54000000p+4 + (-t.rut) * wdot5;
  zp[7] = wdot6 * 0x1.080ddd9000000p+5 * rho_i;
  sum = sum + t.h[6] * wdot6 * 0x1.080ddd9000000p+5 + (-t.rut) * wdot6;
  zp[8] = wdot7 * 0x1.101e302000000p+5 * rho_i;
  sum = sum + t.h[7] * wdot7 * 0x1.101e302000000p+5 + (-t.rut) * wdot7;
  zp[9] = wdot8 * 0x1.c036e20000000p+4 * rho_i;
  sum = sum + t.h[8] * wdot8 * 0x1.c036e20000000p+4 + (-t.rut) * wdot8;
  zp[0] = -sum / (rho * cv);
}

// True when m is the mechanism this file was generated from (every table
// entry the right-hand side reads, bit for bit).
inline bool matches(const izem_mech& m) {
  auto b = [](double x) { unsigned long long u; memcpy(&u, &x, sizeof(u)); return u; };
  if (m.kk != 9 || m.ii != 12 || b(m.ru) != 0x4193d2c630000000ULL) return false;
  if (!(b(m.wt[0]) == 0x3ff020a520000000ULL && b(m.tmid[0]) == 0x408f400000000000ULL && b(m.a[0][0][0]) == 0x4004000000000000ULL && b(m.a[0][0][1]) == 0x3d68d112bff6d580ULL)) return false;
  if (!(b(m.a[0][0][2]) == 0xbce1fa470055807fULL && b(m.a[0][0][3]) == 0x3c4538a620b2373fULL && b(m.a[0][0][4]) == 0xbb91863cffe0b329ULL && b(m.a[0][0][5]) == 0x40d8e06a3bcd35a8ULL)) return false;
  if (!(b(m.a[0][0][6]) == 0xbfdc9673ad546a18ULL && b(m.a[0][1][0]) == 0x40040000015798eeULL && b(m.a[0][1][1]) == 0xbdb961a6ec6a1e45ULL && b(m.a[0][1][2]) == 0x3d1230b4c341c642ULL)) return false;
  if (!(b(m.a[0][1][3]) == 0xbc55d647fbe2e672ULL && b(m.a[0][1][4]) == 0x3b82d244e9510ba2ULL && b(m.a[0][1][5]) == 0x40d8e06a3bcd35a8ULL && b(m.a[0][1][6]) == 0xbfdc9673eed3f77dULL)) return false;
  if (!(b(m.wt[1]) == 0x400020a520000000ULL && b(m.tmid[1]) == 0x408f400000000000ULL && b(m.a[1][0][0]) == 0x4002c130ac9b2911ULL && b(m.a[1][0][1]) == 0x3f8058175d02a941ULL)) return false;
  if (!(b(m.a[1][0][2]) == 0xbef46ca05831775cULL && b(m.a[1][0][3]) == 0x3e55a4c582f87e3dULL && b(m.a[1][0][4]) == 0xbda03862939e564dULL && b(m.a[1][0][5]) == 0xc08caf7b3bfb58d1ULL)) return false;
  if (!(b(m.a[1][0][6]) == 0x3fe5db38496161b4ULL && b(m.a[1][1][0]) == 0x400ab2bf6fecf7e5ULL && b(m.a[1][1][1]) == 0xbf09e6b00cea2ba4ULL && b(m.a[1][1][2]) == 0x3ea0c24d11e93b22ULL)) return false;
  if (!(b(m.a[1][1][3]) == 0xbde8adee4a4b6baeULL && b(m.a[1][1][4]) == 0x3d168bf7de4136dcULL && b(m.a[1][1][5]) == 0xc08db14578e5c4ebULL && b(m.a[1][1][6]) == 0xc009a3e342daf0fdULL)) return false;
  if (!(b(m.wt[2]) == 0x402fffb160000000ULL && b(m.tmid[2]) == 0x408f400000000000ULL && b(m.a[2][0][0]) == 0x4009589c6bdbf12dULL && b(m.a[2][0][1]) == 0xbf6add3ae5787a18ULL)) return false;
  if (!(b(m.a[2][0][2]) == 0x3edbdcef845b6ae0ULL && b(m.a[2][0][3]) == 0xbe3a51e14d5c0503ULL && b(m.a[2][0][4]) == 0x3d82954967e1b470ULL && b(m.a[2][0][5]) == 0x40dc709096bb98c8ULL)) return false;
  if (!(b(m.a[2][0][6]) == 0x40006a5c1702251eULL && b(m.a[2][1][0]) == 0x40048e2c7b5e1a3dULL && b(m.a[2][1][1]) == 0xbf1689a006cdb509ULL && b(m.a[2][1][2]) == 0x3e66855a2fbdda5cULL)) return false;
  if (!(b(m.a[2][1][3]) == 0xbda607823c010ceaULL && b(m.a[2][1][4]) == 0x3cd620b4436bd152ULL && b(m.a[2][1][5]) == 0x40dc88650ff97247ULL && b(m.a[2][1][6]) == 0x40132329ab1f280eULL)) return false;
  if (!(b(m.wt[3]) == 0x403fffb160000000ULL && b(m.tmid[3]) == 0x408f400000000000ULL && b(m.a[3][0][0]) == 0x400e42787ae5fa45ULL && b(m.a[3][0][1]) == 0xbf688c9b66c8c0dfULL)) return false;
  if (!(b(m.a[3][0][2]) == 0x3ee4a6bae1fdae75ULL && b(m.a[3][0][3]) == 0xbe44ca5927ada53cULL && b(m.a[3][0][4]) == 0x3d8c883a18b02bcdULL && b(m.a[3][0][5]) == 0xc0909fc63497b741ULL)) return false;
  if (!(b(m.a[3][0][6]) == 0x400d42eb7e3dc88dULL && b(m.a[3][1][0]) == 0x400a42a332f575b8ULL && b(m.a[3][1][1]) == 0x3f584c851ecf574dULL && b(m.a[3][1][2]) == 0xbea96ee255022a3dULL)) return false;
  if (!(b(m.a[3][1][3]) == 0x3decca1706e20348ULL && b(m.a[3][1][4]) == 0xbd18667712a69c18ULL && b(m.a[3][1][5]) == 0xc09101d4b48d3ae7ULL && b(m.a[3][1][6]) == 0x4015d01bdd004baaULL)) return false;
  if (!(b(m.wt[4]) == 0x403101e302000000ULL && b(m.tmid[4]) == 0x408f400000000000ULL && b(m.a[4][0][0]) == 0x400fefa5c927d1abULL && b(m.a[4][0][1]) == 0xbf63abed86e71c7dULL)) return false;
  if (!(b(m.a[4][0][2]) == 0x3ed35e793e99fbcdULL && b(m.a[4][0][3]) == 0xbe30ab59e9e67441ULL && b(m.a[4][0][4]) == 0x3d77ff6d2c211dd3ULL && b(m.a[4][0][5]) == 0x40ac3e293f290abbULL)) return false;
  if (!(b(m.a[4][0][6]) == 0xbfba9adbdb54f242ULL && b(m.a[4][1][0]) == 0x4008be3be406d029ULL && b(m.a[4][1][1]) == 0x3f41f88fd8e1440eULL && b(m.a[4][1][2]) == 0x3e80faafc0d73234ULL)) return false;
  if (!(b(m.a[4][1][3]) == 0xbdd82ca91827ab6dULL && b(m.a[4][1][4]) == 0x3d0a705cd746f5f8ULL && b(m.a[4][1][5]) == 0x40ae2550624dd2f2ULL && b(m.a[4][1][6]) == 0x4011e82305be85e2ULL)) return false;
  if (!(b(m.wt[5]) == 0x403203ed54000000ULL && b(m.tmid[5]) == 0x408f400000000000ULL && b(m.a[5][0][0]) == 0x4010cb686e536fbfULL && b(m.a[5][0][1]) == 0xbf60aeb63b84c925ULL)) return false;
  if (!(b(m.a[5][0][2]) == 0x3edb593a7c039b70ULL && b(m.a[5][0][3]) == 0xbe37921667072d59ULL && b(m.a[5][0][4]) == 0x3d7f2c47bce627b1ULL && b(m.a[5][0][5]) == 0xc0dd956e8240b780ULL)) return false;
  if (!(b(m.a[5][0][6]) == 0xbfeb2b4597d38a9bULL && b(m.a[5][1][0]) == 0x4008459ddac6e07aULL && b(m.a[5][1][1]) == 0x3f61d553f9364039ULL && b(m.a[5][1][2]) == 0xbe86057d217698d4ULL)) return false;
  if (!(b(m.a[5][1][3]) == 0xbddaacb906a5f7ccULL && b(m.a[5][1][4]) == 0x3d12f01042cd6ffeULL && b(m.a[5][1][5]) == 0xc0dd4d1303afb7e9ULL && b(m.a[5][1][6]) == 0x4013ddf8fb2900aaULL)) return false;
  if (!(b(m.wt[6]) == 0x404080ddd9000000ULL && b(m.tmid[6]) == 0x408f400000000000ULL && b(m.a[6][0][0]) == 0x4011350a899bcaa1ULL && b(m.a[6][0][1]) == 0xbf7373d054674594ULL)) return false;
  if (!(b(m.a[6][0][2]) == 0x3ef62fa28e3a8ea6ULL && b(m.a[6][0][3]) == 0xbe5a110b0905e0fcULL && b(m.a[6][0][4]) == 0x3da46f1288fc5c1cULL && b(m.a[6][0][5]) == 0x40726cedbb59ddc2ULL)) return false;
  if (!(b(m.a[6][0][6]) == 0x400dbbb985c82b7dULL && b(m.a[6][1][0]) == 0x4010119fbbf289f6ULL && b(m.a[6][1][1]) == 0x3f62593e46a1f9dfULL && b(m.a[6][1][2]) == 0xbea5431502070c84ULL)) return false;
  if (!(b(m.a[6][1][3]) == 0x3ddf675fa32f618cULL && b(m.a[6][1][4]) == 0xbd084c80e71ea191ULL && b(m.a[6][1][5]) == 0x405bf6d462c343b7ULL && b(m.a[6][1][6]) == 0x400e47e3a2d22780ULL)) return false;
  if (!(b(m.wt[7]) == 0x404101e302000000ULL && b(m.tmid[7]) == 0x408f400000000000ULL && b(m.a[7][0][0]) == 0x40111abd48f63e0aULL && b(m.a[7][0][1]) == 0xbf41c98643a78c6aULL)) return false;
  if (!(b(m.a[7][0][2]) == 0x3ef18be22e62f026ULL && b(m.a[7][0][3]) == 0xbe572b101d35ae59ULL && b(m.a[7][0][4]) == 0x3da2f72fba30b7c2ULL && b(m.a[7][0][5]) == 0xc0d149a541205bc0ULL)) return false;
  if (!(b(m.a[7][0][6]) == 0x400b7afbe1e3346dULL && b(m.a[7][1][0]) == 0x4010a8f681d1fcb7ULL && b(m.a[7][1][1]) == 0x3f741abe4bc5704bULL && b(m.a[7][1][2]) == 0xbebfe66ae3495cc5ULL)) return false;
  if (!(b(m.a[7][1][3]) == 0x3df981f91177d524ULL && b(m.a[7][1][4]) == 0xbd20353229ef325dULL && b(m.a[7][1][5]) == 0xc0d1717269ad42c4ULL && b(m.a[7][1][6]) == 0x40075449ec074fabULL)) return false;
  if (!(b(m.wt[8]) == 0x403c036e20000000ULL && b(m.tmid[8]) == 0x408f400000000000ULL && b(m.a[8][0][0]) == 0x400a63b0c4588a05ULL && b(m.a[8][0][1]) == 0x3f5712969da04050ULL)) return false;
  if (!(b(m.a[8][0][2]) == 0xbed09f7a2b098bd4ULL && b(m.a[8][0][3]) == 0x3e383ae94da0fe59ULL && b(m.a[8][0][4]) == 0xbd8581526048e0d6ULL && b(m.a[8][0][5]) == 0xc08fe732fec56d5dULL)) return false;
  if (!(b(m.a[8][0][6]) == 0x400f9a5ca29845ddULL && b(m.a[8][1][0]) == 0x400769c23b7952d2ULL && b(m.a[8][1][1]) == 0x3f586106ec5d7fc6ULL && b(m.a[8][1][2]) == 0xbea3132bf1b89c39ULL)) return false;
  if (!(b(m.a[8][1][3]) == 0x3ddbc128a9b8a724ULL && b(m.a[8][1][4]) == 0xbcfe6a15668d1fd9ULL && b(m.a[8][1][5]) == 0xc08cd661b089a027ULL && b(m.a[8][1][6]) == 0x4017ec0f88333fc8ULL)) return false;
  if (!(m.nuk[0][0] == 0 && m.nu[0][0] == -1 && m.nuk[0][1] == 3 && m.nu[0][1] == -1 && m.nuk[0][2] == -1 && m.nu[0][2] == 0 && m.nuk[0][3] == 2 && m.nu[0][3] == 1)) return false;
  if (!(m.nuk[0][4] == 4 && m.nu[0][4] == 1 && m.nuk[0][5] == -1 && m.nu[0][5] == 0 && b(m.par[0][0]) == 0x435f438daa060000ULL && b(m.par[0][1]) == 0xbfe6666666666666ULL)) return false;
  if (!(b(m.par[0][2]) == 0x40c0c6f4493ef159ULL && m.rev[0] == 2 && m.thb[0] == 0 && m.fall[0] == 0 && b(m.lt[0][0]) == 0x0000000000000000ULL && b(m.rlt[0][0]) == 0x0000000000000000ULL && b(m.lt[0][1]) == 0x0000000000000000ULL && b(m.rlt[0][1]) == 0x0000000000000000ULL)) return false;
  if (!(b(m.rpar[0][0]) == 0x42d001d1bf800000ULL && b(m.rpar[0][1]) == 0xbfd0a3d70a3d70a4ULL && b(m.rpar[0][2]) == 0x4051fd705d6afec6ULL && m.nuk[1][0] == 1 && m.nu[1][0] == -1)) return false;
  if (!(m.nuk[1][1] == 2 && m.nu[1][1] == -1 && m.nuk[1][2] == -1 && m.nu[1][2] == 0 && m.nuk[1][3] == 0 && m.nu[1][3] == 1 && m.nuk[1][4] == 4 && m.nu[1][4] == 1)) return false;
  if (!(m.nuk[1][5] == -1 && m.nu[1][5] == 0 && b(m.par[1][0]) == 0x40e8b50000000000ULL && b(m.par[1][1]) == 0x40055c28f5c28f5cULL && b(m.par[1][2]) == 0x40a8bb78dad5b973ULL)) return false;
  if (!(m.rev[1] == 2 && m.thb[1] == 0 && m.fall[1] == 0 && b(m.lt[1][0]) == 0x0000000000000000ULL && b(m.rlt[1][0]) == 0x0000000000000000ULL && b(m.lt[1][1]) == 0x0000000000000000ULL && b(m.rlt[1][1]) == 0x0000000000000000ULL && b(m.rpar[1][0]) == 0x40dd970000000000ULL)) return false;
  if (!(b(m.rpar[1][1]) == 0x40050a3d70a3d70aULL && b(m.rpar[1][2]) == 0x40a3072327bb03a1ULL && m.nuk[2][0] == 1 && m.nu[2][0] == -1 && m.nuk[2][1] == 4 && m.nu[2][1] == -1)) return false;
  if (!(m.nuk[2][2] == -1 && m.nu[2][2] == 0 && m.nuk[2][3] == 0 && m.nu[2][3] == 1 && m.nuk[2][4] == 5 && m.nu[2][4] == 1 && m.nuk[2][5] == -1 && m.nu[2][5] == 0)) return false;
  if (!(b(m.par[2][0]) == 0x41d16f3220000000ULL && b(m.par[2][1]) == 0x3ff4cccccccccccdULL && b(m.par[2][2]) == 0x409c94c533be761cULL && m.rev[2] == 2 && m.thb[2] == 0 && m.fall[2] == 0)) return false;
  if (!(b(m.lt[2][0]) == 0x0000000000000000ULL && b(m.rlt[2][0]) == 0x0000000000000000ULL && b(m.lt[2][1]) == 0x0000000000000000ULL && b(m.rlt[2][1]) == 0x0000000000000000ULL && b(m.rpar[2][0]) == 0x4207d78400000000ULL && b(m.rpar[2][1]) == 0x3ff30a3d70a3d70aULL)) return false;
  if (!(b(m.rpar[2][2]) == 0x40c2611369490098ULL && m.nuk[3][0] == 0 && m.nu[3][0] == -1 && m.nuk[3][1] == 3 && m.nu[3][1] == -1 && m.nuk[3][2] == -1 && m.nu[3][2] == 0)) return false;
  if (!(m.nuk[3][3] == 6 && m.nu[3][3] == 1 && m.nuk[3][4] == -1 && m.nu[3][4] == 0 && m.nuk[3][5] == -1 && m.nu[3][5] == 0 && b(m.par[3][0]) == 0x4290eaa664900000ULL)) return false;
  if (!(b(m.par[3][1]) == 0x3fdc28f5c28f5c29ULL && b(m.par[3][2]) == 0x0000000000000000ULL && m.rev[3] == 0 && m.thb[3] == 1 && m.fall[3] == 3 && b(m.lt[3][0]) == 0x0000000000000000ULL && b(m.rlt[3][0]) == 0x0000000000000000ULL)) return false;
  if (!(b(m.lt[3][1]) == 0x0000000000000000ULL && b(m.rlt[3][1]) == 0x0000000000000000ULL && b(m.eff[3][0]) == 0x3ff0000000000000ULL && b(m.eff[3][1]) == 0x4004000000000000ULL && b(m.eff[3][2]) == 0x3ff0000000000000ULL)) return false;
  if (!(b(m.eff[3][3]) == 0x3ff0000000000000ULL && b(m.eff[3][4]) == 0x3ff0000000000000ULL && b(m.eff[3][5]) == 0x4030000000000000ULL && b(m.eff[3][6]) == 0x3ff0000000000000ULL)) return false;
  if (!(b(m.eff[3][7]) == 0x3ff0000000000000ULL && b(m.eff[3][8]) == 0x3ff0000000000000ULL && m.kfal[3] == 0 && b(m.low[3][0]) == 0x4408efc84ad0c7b0ULL)) return false;
  if (!(b(m.low[3][1]) == 0xbff6666666666666ULL && b(m.low[3][2]) == 0x0000000000000000ULL && b(m.troe[3][0]) == 0x3fe0000000000000ULL && b(m.troe[3][1]) == 0x39b4484bfeebc2a0ULL)) return false;
  if (!(b(m.troe[3][2]) == 0x46293e5939a08ceaULL && m.nuk[4][0] == 0 && m.nu[4][0] == -1 && m.nuk[4][1] == 6 && m.nu[4][1] == -1 && m.nuk[4][2] == -1 && m.nu[4][2] == 0)) return false;
  if (!(m.nuk[4][3] == 4 && m.nu[4][3] == 2 && m.nuk[4][4] == -1 && m.nu[4][4] == 0 && m.nuk[4][5] == -1 && m.nu[4][5] == 0 && b(m.par[4][0]) == 0x42d0191a36680000ULL)) return false;
  if (!(b(m.par[4][1]) == 0x0000000000000000ULL && b(m.par[4][2]) == 0x40627e432c1d6dbcULL && m.rev[4] == 0 && m.thb[4] == 0 && m.fall[4] == 0 && b(m.lt[4][0]) == 0x0000000000000000ULL && b(m.rlt[4][0]) == 0x0000000000000000ULL)) return false;
  if (!(b(m.lt[4][1]) == 0x0000000000000000ULL && b(m.rlt[4][1]) == 0x0000000000000000ULL && m.nuk[5][0] == 0 && m.nu[5][0] == -1 && m.nuk[5][1] == 6 && m.nu[5][1] == -1 && m.nuk[5][2] == -1 && m.nu[5][2] == 0)) return false;
  if (!(m.nuk[5][3] == 1 && m.nu[5][3] == 1 && m.nuk[5][4] == 3 && m.nu[5][4] == 1 && m.nuk[5][5] == -1 && m.nu[5][5] == 0 && b(m.par[5][0]) == 0x42ae31fa34e00000ULL)) return false;
  if (!(b(m.par[5][1]) == 0x0000000000000000ULL && b(m.par[5][2]) == 0x4079da4e3b0f0481ULL && m.rev[5] == 2 && m.thb[5] == 0 && m.fall[5] == 0 && b(m.lt[5][0]) == 0x0000000000000000ULL && b(m.rlt[5][0]) == 0x0000000000000000ULL)) return false;
  if (!(b(m.lt[5][1]) == 0x0000000000000000ULL && b(m.rlt[5][1]) == 0x0000000000000000ULL && b(m.rpar[5][0]) == 0x42839283f4a00000ULL && b(m.rpar[5][1]) == 0x3fd70a3d70a3d70aULL && b(m.rpar[5][2]) == 0x40db3c1120ab0336ULL)) return false;
  if (!(m.nuk[6][0] == 4 && m.nu[6][0] == -1 && m.nuk[6][1] == 6 && m.nu[6][1] == -1 && m.nuk[6][2] == -1 && m.nu[6][2] == 0 && m.nuk[6][3] == 3 && m.nu[6][3] == 1)) return false;
  if (!(m.nuk[6][4] == 5 && m.nu[6][4] == 1 && m.nuk[6][5] == -1 && m.nu[6][5] == 0 && b(m.par[6][0]) == 0x42ba48ce3be80000ULL && b(m.par[6][1]) == 0x0000000000000000ULL)) return false;
  if (!(b(m.par[6][2]) == 0xc06f4328690d2d50ULL && m.rev[6] == 0 && m.thb[6] == 0 && m.fall[6] == 0 && b(m.lt[6][0]) == 0x0000000000000000ULL && b(m.rlt[6][0]) == 0x0000000000000000ULL && b(m.lt[6][1]) == 0x0000000000000000ULL && b(m.rlt[6][1]) == 0x0000000000000000ULL)) return false;
  if (!(m.nuk[7][0] == 0 && m.nu[7][0] == -1 && m.nuk[7][1] == 4 && m.nu[7][1] == -1 && m.nuk[7][2] == -1 && m.nu[7][2] == 0 && m.nuk[7][3] == 5 && m.nu[7][3] == 1)) return false;
  if (!(m.nuk[7][4] == -1 && m.nu[7][4] == 0 && m.nuk[7][5] == -1 && m.nu[7][5] == 0 && b(m.par[7][0]) == 0x44a0f0cf064dd592ULL && b(m.par[7][1]) == 0xc000000000000000ULL)) return false;
  if (!(b(m.par[7][2]) == 0x0000000000000000ULL && m.rev[7] == 2 && m.thb[7] == 1 && m.fall[7] == 0 && b(m.lt[7][0]) == 0x0000000000000000ULL && b(m.rlt[7][0]) == 0x0000000000000000ULL && b(m.lt[7][1]) == 0x0000000000000000ULL && b(m.rlt[7][1]) == 0x0000000000000000ULL)) return false;
  if (!(b(m.rpar[7][0]) == 0x44b5cfa424ea9c92ULL && b(m.rpar[7][1]) == 0xbffc000000000000ULL && b(m.rpar[7][2]) == 0x40ed22edd4d65d8eULL && b(m.eff[7][0]) == 0x3ff0000000000000ULL)) return false;
  if (!(b(m.eff[7][1]) == 0x4004000000000000ULL && b(m.eff[7][2]) == 0x3ff0000000000000ULL && b(m.eff[7][3]) == 0x3ff0000000000000ULL && b(m.eff[7][4]) == 0x3ff0000000000000ULL)) return false;
  if (!(b(m.eff[7][5]) == 0x4028000000000000ULL && b(m.eff[7][6]) == 0x3ff0000000000000ULL && b(m.eff[7][7]) == 0x3ff0000000000000ULL && b(m.eff[7][8]) == 0x3ff0000000000000ULL)) return false;
  if (!(m.nuk[8][0] == 0 && m.nu[8][0] == -2 && m.nuk[8][1] == -1 && m.nu[8][1] == 0 && m.nuk[8][2] == -1 && m.nu[8][2] == 0 && m.nuk[8][3] == 1 && m.nu[8][3] == 1)) return false;
  if (!(m.nuk[8][4] == -1 && m.nu[8][4] == 0 && m.nuk[8][5] == -1 && m.nu[8][5] == 0 && b(m.par[8][0]) == 0x43b20a871cc00200ULL && b(m.par[8][1]) == 0xbff0000000000000ULL)) return false;
  if (!(b(m.par[8][2]) == 0x0000000000000000ULL && m.rev[8] == 2 && m.thb[8] == 1 && m.fall[8] == 0 && b(m.lt[8][0]) == 0x0000000000000000ULL && b(m.rlt[8][0]) == 0x0000000000000000ULL && b(m.lt[8][1]) == 0x0000000000000000ULL && b(m.rlt[8][1]) == 0x0000000000000000ULL)) return false;
  if (!(b(m.rpar[8][0]) == 0x4390e0198eaee000ULL && b(m.rpar[8][1]) == 0xbfe4cccccccccccdULL && b(m.rpar[8][2]) == 0x40e96e5d98de8289ULL && b(m.eff[8][0]) == 0x3ff0000000000000ULL)) return false;
  if (!(b(m.eff[8][1]) == 0x4004000000000000ULL && b(m.eff[8][2]) == 0x3ff0000000000000ULL && b(m.eff[8][3]) == 0x3ff0000000000000ULL && b(m.eff[8][4]) == 0x3ff0000000000000ULL)) return false;
  if (!(b(m.eff[8][5]) == 0x4028000000000000ULL && b(m.eff[8][6]) == 0x3ff0000000000000ULL && b(m.eff[8][7]) == 0x3ff0000000000000ULL && b(m.eff[8][8]) == 0x3ff0000000000000ULL)) return false;
  if (!(m.nuk[9][0] == 6 && m.nu[9][0] == -2 && m.nuk[9][1] == -1 && m.nu[9][1] == 0 && m.nuk[9][2] == -1 && m.nu[9][2] == 0 && m.nuk[9][3] == 3 && m.nu[9][3] == 1)) return false;
  if (!(m.nuk[9][4] == 7 && m.nu[9][4] == 1 && m.nuk[9][5] == -1 && m.nu[9][5] == 0 && b(m.par[9][0]) == 0x4285f93037c00000ULL && b(m.par[9][1]) == 0x0000000000000000ULL)) return false;
  if (!(b(m.par[9][2]) == 0x4085dbc4f266b3c5ULL && m.rev[9] == 0 && m.thb[9] == 0 && m.fall[9] == 0 && b(m.lt[9][0]) == 0x0000000000000000ULL && b(m.rlt[9][0]) == 0x0000000000000000ULL && b(m.lt[9][1]) == 0x0000000000000000ULL && b(m.rlt[9][1]) == 0x0000000000000000ULL)) return false;
  if (!(m.nuk[10][0] == 1 && m.nu[10][0] == -1 && m.nuk[10][1] == 6 && m.nu[10][1] == -1 && m.nuk[10][2] == -1 && m.nu[10][2] == 0 && m.nuk[10][3] == 0 && m.nu[10][3] == 1)) return false;
  if (!(m.nuk[10][4] == 7 && m.nu[10][4] == 1 && m.nuk[10][5] == -1 && m.nu[10][5] == 0 && b(m.par[10][0]) == 0x4242dbf9ea000000ULL && b(m.par[10][1]) == 0x3fe3851eb851eb85ULL)) return false;
  if (!(b(m.par[10][2]) == 0x40c784fcc6a9ac05ULL && m.rev[10] == 0 && m.thb[10] == 0 && m.fall[10] == 0 && b(m.lt[10][0]) == 0x0000000000000000ULL && b(m.rlt[10][0]) == 0x0000000000000000ULL && b(m.lt[10][1]) == 0x0000000000000000ULL && b(m.rlt[10][1]) == 0x0000000000000000ULL)) return false;
  if (!(m.nuk[11][0] == 7 && m.nu[11][0] == -1 && m.nuk[11][1] == -1 && m.nu[11][1] == 0 && m.nuk[11][2] == -1 && m.nu[11][2] == 0 && m.nuk[11][3] == 4 && m.nu[11][3] == 2)) return false;
  if (!(m.nuk[11][4] == -1 && m.nu[11][4] == 0 && m.nuk[11][5] == -1 && m.nu[11][5] == 0 && b(m.par[11][0]) == 0x43f6b99192fbb3c0ULL && b(m.par[11][1]) == 0xbff63d70a3d70a3dULL)) return false;
  if (!(b(m.par[11][2]) == 0x40d93845131294f1ULL && m.rev[11] == 0 && m.thb[11] == 1 && m.fall[11] == 4 && b(m.lt[11][0]) == 0x0000000000000000ULL && b(m.rlt[11][0]) == 0x0000000000000000ULL && b(m.lt[11][1]) == 0x0000000000000000ULL && b(m.rlt[11][1]) == 0x0000000000000000ULL)) return false;
  if (!(b(m.eff[11][0]) == 0x3ff0000000000000ULL && b(m.eff[11][1]) == 0x4004000000000000ULL && b(m.eff[11][2]) == 0x3ff0000000000000ULL && b(m.eff[11][3]) == 0x3ff0000000000000ULL)) return false;
  if (!(b(m.eff[11][4]) == 0x3ff0000000000000ULL && b(m.eff[11][5]) == 0x4018000000000000ULL && b(m.eff[11][6]) == 0x3ff0000000000000ULL && b(m.eff[11][7]) == 0x3ff0000000000000ULL)) return false;
  if (!(b(m.eff[11][8]) == 0x3ff0000000000000ULL && m.kfal[11] == 0 && b(m.low[11][0]) == 0x44e592a7a2071df8ULL && b(m.low[11][1]) == 0xbffe666666666666ULL)) return false;
  if (!(b(m.low[11][2]) == 0x40d8626719ec5abbULL && b(m.troe[11][0]) == 0x3fe7851eb851eb85ULL && b(m.troe[11][1]) == 0x4057800000000000ULL && b(m.troe[11][2]) == 0x409b700000000000ULL)) return false;
  if (!(b(m.troe[11][3]) == 0x40b43e0000000000ULL)) return false;
  return true;
}

}  // namespace chem_gen
