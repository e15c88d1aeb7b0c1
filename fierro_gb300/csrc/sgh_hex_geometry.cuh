// GENERATED by gen_hex_geometry.py from sgh_hex.h -- do not edit.
// Straight-line hex geometry; see the generator's docstring for the exactness argument.
#pragma once

// Separately rounded product and sum, also where the unit contracts (FIERRO_FMA=1).
#if FIERRO_FMA
#define FX_MUL(a, b) __dmul_rn((a), (b))
#define FX_ADD(a, b) __dadd_rn((a), (b))
#else
#define FX_MUL(a, b) ((a) * (b))
#define FX_ADD(a, b) ((a) + (b))
#endif

// In: x,y,z,u,v,w[8] (node lids 0..7).  Out: vol; bmat rows lid*3+dim at
// bmat[row*ne + e]; Sx,Sy,Sz = sum_p u_p B(p,0), v_p B(p,1), w_p B(p,2) (p order).
__device__ __forceinline__ void hex_geometry(const double* __restrict__ x, const double* __restrict__ y,
    const double* __restrict__ z, const double* __restrict__ u, const double* __restrict__ v,
    const double* __restrict__ w, double* __restrict__ bmat, int ne, int e, double& vol,
    double& Sx, double& Sy, double& Sz) {
  const double twelth = 1. / 12.;
  {  // component 0: O = y, I = z
    const double cm0 = (((-z[2] - z[3]) + z[4]) + z[5]);  // pair (0,1)
    const double cm1 = (z[1] - z[3]);  // pair (0,2)
    const double cm2 = (((z[1] + z[2]) - z[4]) - z[7]);  // pair (0,3)
    const double cm3 = (((-z[1] + z[3]) - z[5]) + z[7]);  // pair (0,4)
    const double cm4 = (-z[1] + z[4]);  // pair (0,5)
    const double cm5 = (z[3] - z[4]);  // pair (0,7)
    const double cm6 = (((-z[0] - z[3]) + z[5]) + z[6]);  // pair (1,2)
    const double cm7 = (-z[0] + z[2]);  // pair (1,3)
    const double cm8 = (z[0] - z[5]);  // pair (1,4)
    const double cm9 = (((z[0] - z[2]) + z[4]) - z[6]);  // pair (1,5)
    const double cm10 = (-z[2] + z[5]);  // pair (1,6)
    const double cm11 = (((-z[0] - z[1]) + z[6]) + z[7]);  // pair (2,3)
    const double cm12 = (z[1] - z[6]);  // pair (2,5)
    const double cm13 = (((z[1] - z[3]) + z[5]) - z[7]);  // pair (2,6)
    const double cm14 = (-z[3] + z[6]);  // pair (2,7)
    const double cm15 = (-z[0] + z[7]);  // pair (3,4)
    const double cm16 = (z[2] - z[7]);  // pair (3,6)
    const double cm17 = (((-z[0] + z[2]) - z[4]) + z[6]);  // pair (3,7)
    const double cm18 = (((-z[0] - z[1]) + z[6]) + z[7]);  // pair (4,5)
    const double cm19 = (-z[5] + z[7]);  // pair (4,6)
    const double cm20 = (((z[0] + z[3]) - z[5]) - z[6]);  // pair (4,7)
    const double cm21 = (((-z[1] - z[2]) + z[4]) + z[7]);  // pair (5,6)
    const double cm22 = (z[4] - z[6]);  // pair (5,7)
    const double cm23 = (((-z[2] - z[3]) + z[4]) + z[5]);  // pair (6,7)
    const double pr0_0 = FX_MUL(y[1], cm0);
    const double pr0_1 = FX_MUL(y[2], cm1);
    const double pr0_2 = FX_MUL(y[3], cm2);
    const double pr0_3 = FX_MUL(y[4], cm3);
    const double pr0_4 = FX_MUL(y[5], cm4);
    const double pr0_5 = FX_MUL(y[7], cm5);
    const double pr1_0 = FX_MUL(y[0], (-cm0));
    const double pr1_1 = FX_MUL(y[2], cm6);
    const double pr1_2 = FX_MUL(y[3], cm7);
    const double pr1_3 = FX_MUL(y[4], cm8);
    const double pr1_4 = FX_MUL(y[5], cm9);
    const double pr1_5 = FX_MUL(y[6], cm10);
    const double pr2_0 = FX_MUL(y[0], (-cm1));
    const double pr2_1 = FX_MUL(y[1], (-cm6));
    const double pr2_2 = FX_MUL(y[3], cm11);
    const double pr2_3 = FX_MUL(y[5], cm12);
    const double pr2_4 = FX_MUL(y[6], cm13);
    const double pr2_5 = FX_MUL(y[7], cm14);
    const double pr3_0 = FX_MUL(y[0], (-cm2));
    const double pr3_1 = FX_MUL(y[1], (-cm7));
    const double pr3_2 = FX_MUL(y[2], (-cm11));
    const double pr3_3 = FX_MUL(y[4], cm15);
    const double pr3_4 = FX_MUL(y[6], cm16);
    const double pr3_5 = FX_MUL(y[7], cm17);
    const double pr4_0 = FX_MUL(y[0], (-cm3));
    const double pr4_1 = FX_MUL(y[1], (-cm8));
    const double pr4_2 = FX_MUL(y[3], (-cm15));
    const double pr4_3 = FX_MUL(y[5], cm18);
    const double pr4_4 = FX_MUL(y[6], cm19);
    const double pr4_5 = FX_MUL(y[7], cm20);
    const double pr5_0 = FX_MUL(y[0], (-cm4));
    const double pr5_1 = FX_MUL(y[1], (-cm9));
    const double pr5_2 = FX_MUL(y[2], (-cm12));
    const double pr5_3 = FX_MUL(y[4], (-cm18));
    const double pr5_4 = FX_MUL(y[6], cm21);
    const double pr5_5 = FX_MUL(y[7], cm22);
    const double pr6_0 = FX_MUL(y[1], (-cm10));
    const double pr6_1 = FX_MUL(y[2], (-cm13));
    const double pr6_2 = FX_MUL(y[3], (-cm16));
    const double pr6_3 = FX_MUL(y[4], (-cm19));
    const double pr6_4 = FX_MUL(y[5], (-cm21));
    const double pr6_5 = FX_MUL(y[7], cm23);
    const double pr7_0 = FX_MUL(y[0], (-cm5));
    const double pr7_1 = FX_MUL(y[2], (-cm14));
    const double pr7_2 = FX_MUL(y[3], (-cm17));
    const double pr7_3 = FX_MUL(y[4], (-cm20));
    const double pr7_4 = FX_MUL(y[5], (-cm22));
    const double pr7_5 = FX_MUL(y[6], (-cm23));
    const double vi0 = FX_MUL(x[1], FX_ADD(FX_ADD(FX_ADD(FX_ADD(FX_ADD(pr1_2, pr1_3), pr1_0), pr1_5), pr1_4), pr1_1));
    const double vi1 = FX_MUL(x[7], FX_ADD(FX_ADD(FX_ADD(FX_ADD(FX_ADD(pr7_0, pr7_5), pr7_1), pr7_2), pr7_4), pr7_3));
    const double vi2 = FX_MUL(x[3], FX_ADD(FX_ADD(FX_ADD(FX_ADD(FX_ADD(pr3_1, pr3_5), pr3_4), pr3_2), pr3_3), pr3_0));
    const double vi3 = FX_MUL(x[5], FX_ADD(FX_ADD(FX_ADD(FX_ADD(FX_ADD(pr5_0, pr5_5), pr5_2), pr5_1), pr5_3), pr5_4));
    const double vi4 = FX_MUL(x[6], FX_ADD(FX_ADD(FX_ADD(FX_ADD(FX_ADD(pr6_0, pr6_5), pr6_4), pr6_3), pr6_2), pr6_1));
    const double vi5 = FX_MUL(x[0], FX_ADD(FX_ADD(FX_ADD(FX_ADD(FX_ADD(pr0_1, pr0_5), pr0_4), pr0_0), pr0_2), pr0_3));
    const double vi6 = FX_MUL(x[2], FX_ADD(FX_ADD(FX_ADD(FX_ADD(FX_ADD(pr2_0, pr2_3), pr2_1), pr2_5), pr2_4), pr2_2));
    const double vi7 = FX_MUL(x[4], FX_ADD(FX_ADD(FX_ADD(FX_ADD(FX_ADD(pr4_1, pr4_5), pr4_2), pr4_0), pr4_4), pr4_3));
    vol = FX_MUL(FX_ADD(FX_ADD(FX_ADD(FX_ADD(FX_ADD(FX_ADD(FX_ADD(vi0, vi1), vi2), vi3), vi4), vi5), vi6), vi7), twelth);
    const double b0 = (((((pr0_0 + pr0_1) + pr0_2) + pr0_3) + pr0_4) + pr0_5) * twelth;
    bmat[(size_t)0 * ne + e] = b0;
    Sx = u[0] * b0;
    const double b1 = (((((pr1_0 + pr1_1) + pr1_2) + pr1_3) + pr1_4) + pr1_5) * twelth;
    bmat[(size_t)3 * ne + e] = b1;
    Sx = Sx + u[1] * b1;
    const double b2 = (((((pr2_0 + pr2_1) + pr2_2) + pr2_3) + pr2_4) + pr2_5) * twelth;
    bmat[(size_t)6 * ne + e] = b2;
    Sx = Sx + u[2] * b2;
    const double b3 = (((((pr3_0 + pr3_1) + pr3_2) + pr3_3) + pr3_4) + pr3_5) * twelth;
    bmat[(size_t)9 * ne + e] = b3;
    Sx = Sx + u[3] * b3;
    const double b4 = (((((pr4_0 + pr4_1) + pr4_2) + pr4_3) + pr4_4) + pr4_5) * twelth;
    bmat[(size_t)12 * ne + e] = b4;
    Sx = Sx + u[4] * b4;
    const double b5 = (((((pr5_0 + pr5_1) + pr5_2) + pr5_3) + pr5_4) + pr5_5) * twelth;
    bmat[(size_t)15 * ne + e] = b5;
    Sx = Sx + u[5] * b5;
    const double b6 = (((((pr6_0 + pr6_1) + pr6_2) + pr6_3) + pr6_4) + pr6_5) * twelth;
    bmat[(size_t)18 * ne + e] = b6;
    Sx = Sx + u[6] * b6;
    const double b7 = (((((pr7_0 + pr7_1) + pr7_2) + pr7_3) + pr7_4) + pr7_5) * twelth;
    bmat[(size_t)21 * ne + e] = b7;
    Sx = Sx + u[7] * b7;
  }
  {  // component 1: O = z, I = x
    const double cm0 = (((-x[2] - x[3]) + x[4]) + x[5]);  // pair (0,1)
    const double cm1 = (x[1] - x[3]);  // pair (0,2)
    const double cm2 = (((x[1] + x[2]) - x[4]) - x[7]);  // pair (0,3)
    const double cm3 = (((-x[1] + x[3]) - x[5]) + x[7]);  // pair (0,4)
    const double cm4 = (-x[1] + x[4]);  // pair (0,5)
    const double cm5 = (x[3] - x[4]);  // pair (0,7)
    const double cm6 = (((-x[0] - x[3]) + x[5]) + x[6]);  // pair (1,2)
    const double cm7 = (-x[0] + x[2]);  // pair (1,3)
    const double cm8 = (x[0] - x[5]);  // pair (1,4)
    const double cm9 = (((x[0] - x[2]) + x[4]) - x[6]);  // pair (1,5)
    const double cm10 = (-x[2] + x[5]);  // pair (1,6)
    const double cm11 = (((-x[0] - x[1]) + x[6]) + x[7]);  // pair (2,3)
    const double cm12 = (x[1] - x[6]);  // pair (2,5)
    const double cm13 = (((x[1] - x[3]) + x[5]) - x[7]);  // pair (2,6)
    const double cm14 = (-x[3] + x[6]);  // pair (2,7)
    const double cm15 = (-x[0] + x[7]);  // pair (3,4)
    const double cm16 = (x[2] - x[7]);  // pair (3,6)
    const double cm17 = (((-x[0] + x[2]) - x[4]) + x[6]);  // pair (3,7)
    const double cm18 = (((-x[0] - x[1]) + x[6]) + x[7]);  // pair (4,5)
    const double cm19 = (-x[5] + x[7]);  // pair (4,6)
    const double cm20 = (((x[0] + x[3]) - x[5]) - x[6]);  // pair (4,7)
    const double cm21 = (((-x[1] - x[2]) + x[4]) + x[7]);  // pair (5,6)
    const double cm22 = (x[4] - x[6]);  // pair (5,7)
    const double cm23 = (((-x[2] - x[3]) + x[4]) + x[5]);  // pair (6,7)
    const double pr0_0 = z[1] * cm0;
    const double pr0_1 = z[2] * cm1;
    const double pr0_2 = z[3] * cm2;
    const double pr0_3 = z[4] * cm3;
    const double pr0_4 = z[5] * cm4;
    const double pr0_5 = z[7] * cm5;
    const double pr1_0 = z[0] * (-cm0);
    const double pr1_1 = z[2] * cm6;
    const double pr1_2 = z[3] * cm7;
    const double pr1_3 = z[4] * cm8;
    const double pr1_4 = z[5] * cm9;
    const double pr1_5 = z[6] * cm10;
    const double pr2_0 = z[0] * (-cm1);
    const double pr2_1 = z[1] * (-cm6);
    const double pr2_2 = z[3] * cm11;
    const double pr2_3 = z[5] * cm12;
    const double pr2_4 = z[6] * cm13;
    const double pr2_5 = z[7] * cm14;
    const double pr3_0 = z[0] * (-cm2);
    const double pr3_1 = z[1] * (-cm7);
    const double pr3_2 = z[2] * (-cm11);
    const double pr3_3 = z[4] * cm15;
    const double pr3_4 = z[6] * cm16;
    const double pr3_5 = z[7] * cm17;
    const double pr4_0 = z[0] * (-cm3);
    const double pr4_1 = z[1] * (-cm8);
    const double pr4_2 = z[3] * (-cm15);
    const double pr4_3 = z[5] * cm18;
    const double pr4_4 = z[6] * cm19;
    const double pr4_5 = z[7] * cm20;
    const double pr5_0 = z[0] * (-cm4);
    const double pr5_1 = z[1] * (-cm9);
    const double pr5_2 = z[2] * (-cm12);
    const double pr5_3 = z[4] * (-cm18);
    const double pr5_4 = z[6] * cm21;
    const double pr5_5 = z[7] * cm22;
    const double pr6_0 = z[1] * (-cm10);
    const double pr6_1 = z[2] * (-cm13);
    const double pr6_2 = z[3] * (-cm16);
    const double pr6_3 = z[4] * (-cm19);
    const double pr6_4 = z[5] * (-cm21);
    const double pr6_5 = z[7] * cm23;
    const double pr7_0 = z[0] * (-cm5);
    const double pr7_1 = z[2] * (-cm14);
    const double pr7_2 = z[3] * (-cm17);
    const double pr7_3 = z[4] * (-cm20);
    const double pr7_4 = z[5] * (-cm22);
    const double pr7_5 = z[6] * (-cm23);
    const double b0 = (((((pr0_0 + pr0_1) + pr0_2) + pr0_3) + pr0_4) + pr0_5) * twelth;
    bmat[(size_t)1 * ne + e] = b0;
    Sy = v[0] * b0;
    const double b1 = (((((pr1_0 + pr1_1) + pr1_2) + pr1_3) + pr1_4) + pr1_5) * twelth;
    bmat[(size_t)4 * ne + e] = b1;
    Sy = Sy + v[1] * b1;
    const double b2 = (((((pr2_0 + pr2_1) + pr2_2) + pr2_3) + pr2_4) + pr2_5) * twelth;
    bmat[(size_t)7 * ne + e] = b2;
    Sy = Sy + v[2] * b2;
    const double b3 = (((((pr3_0 + pr3_1) + pr3_2) + pr3_3) + pr3_4) + pr3_5) * twelth;
    bmat[(size_t)10 * ne + e] = b3;
    Sy = Sy + v[3] * b3;
    const double b4 = (((((pr4_0 + pr4_1) + pr4_2) + pr4_3) + pr4_4) + pr4_5) * twelth;
    bmat[(size_t)13 * ne + e] = b4;
    Sy = Sy + v[4] * b4;
    const double b5 = (((((pr5_0 + pr5_1) + pr5_2) + pr5_3) + pr5_4) + pr5_5) * twelth;
    bmat[(size_t)16 * ne + e] = b5;
    Sy = Sy + v[5] * b5;
    const double b6 = (((((pr6_0 + pr6_1) + pr6_2) + pr6_3) + pr6_4) + pr6_5) * twelth;
    bmat[(size_t)19 * ne + e] = b6;
    Sy = Sy + v[6] * b6;
    const double b7 = (((((pr7_0 + pr7_1) + pr7_2) + pr7_3) + pr7_4) + pr7_5) * twelth;
    bmat[(size_t)22 * ne + e] = b7;
    Sy = Sy + v[7] * b7;
  }
  {  // component 2: O = x, I = y
    const double cm0 = (((-y[2] - y[3]) + y[4]) + y[5]);  // pair (0,1)
    const double cm1 = (y[1] - y[3]);  // pair (0,2)
    const double cm2 = (((y[1] + y[2]) - y[4]) - y[7]);  // pair (0,3)
    const double cm3 = (((-y[1] + y[3]) - y[5]) + y[7]);  // pair (0,4)
    const double cm4 = (-y[1] + y[4]);  // pair (0,5)
    const double cm5 = (y[3] - y[4]);  // pair (0,7)
    const double cm6 = (((-y[0] - y[3]) + y[5]) + y[6]);  // pair (1,2)
    const double cm7 = (-y[0] + y[2]);  // pair (1,3)
    const double cm8 = (y[0] - y[5]);  // pair (1,4)
    const double cm9 = (((y[0] - y[2]) + y[4]) - y[6]);  // pair (1,5)
    const double cm10 = (-y[2] + y[5]);  // pair (1,6)
    const double cm11 = (((-y[0] - y[1]) + y[6]) + y[7]);  // pair (2,3)
    const double cm12 = (y[1] - y[6]);  // pair (2,5)
    const double cm13 = (((y[1] - y[3]) + y[5]) - y[7]);  // pair (2,6)
    const double cm14 = (-y[3] + y[6]);  // pair (2,7)
    const double cm15 = (-y[0] + y[7]);  // pair (3,4)
    const double cm16 = (y[2] - y[7]);  // pair (3,6)
    const double cm17 = (((-y[0] + y[2]) - y[4]) + y[6]);  // pair (3,7)
    const double cm18 = (((-y[0] - y[1]) + y[6]) + y[7]);  // pair (4,5)
    const double cm19 = (-y[5] + y[7]);  // pair (4,6)
    const double cm20 = (((y[0] + y[3]) - y[5]) - y[6]);  // pair (4,7)
    const double cm21 = (((-y[1] - y[2]) + y[4]) + y[7]);  // pair (5,6)
    const double cm22 = (y[4] - y[6]);  // pair (5,7)
    const double cm23 = (((-y[2] - y[3]) + y[4]) + y[5]);  // pair (6,7)
    const double pr0_0 = x[1] * cm0;
    const double pr0_1 = x[2] * cm1;
    const double pr0_2 = x[3] * cm2;
    const double pr0_3 = x[4] * cm3;
    const double pr0_4 = x[5] * cm4;
    const double pr0_5 = x[7] * cm5;
    const double pr1_0 = x[0] * (-cm0);
    const double pr1_1 = x[2] * cm6;
    const double pr1_2 = x[3] * cm7;
    const double pr1_3 = x[4] * cm8;
    const double pr1_4 = x[5] * cm9;
    const double pr1_5 = x[6] * cm10;
    const double pr2_0 = x[0] * (-cm1);
    const double pr2_1 = x[1] * (-cm6);
    const double pr2_2 = x[3] * cm11;
    const double pr2_3 = x[5] * cm12;
    const double pr2_4 = x[6] * cm13;
    const double pr2_5 = x[7] * cm14;
    const double pr3_0 = x[0] * (-cm2);
    const double pr3_1 = x[1] * (-cm7);
    const double pr3_2 = x[2] * (-cm11);
    const double pr3_3 = x[4] * cm15;
    const double pr3_4 = x[6] * cm16;
    const double pr3_5 = x[7] * cm17;
    const double pr4_0 = x[0] * (-cm3);
    const double pr4_1 = x[1] * (-cm8);
    const double pr4_2 = x[3] * (-cm15);
    const double pr4_3 = x[5] * cm18;
    const double pr4_4 = x[6] * cm19;
    const double pr4_5 = x[7] * cm20;
    const double pr5_0 = x[0] * (-cm4);
    const double pr5_1 = x[1] * (-cm9);
    const double pr5_2 = x[2] * (-cm12);
    const double pr5_3 = x[4] * (-cm18);
    const double pr5_4 = x[6] * cm21;
    const double pr5_5 = x[7] * cm22;
    const double pr6_0 = x[1] * (-cm10);
    const double pr6_1 = x[2] * (-cm13);
    const double pr6_2 = x[3] * (-cm16);
    const double pr6_3 = x[4] * (-cm19);
    const double pr6_4 = x[5] * (-cm21);
    const double pr6_5 = x[7] * cm23;
    const double pr7_0 = x[0] * (-cm5);
    const double pr7_1 = x[2] * (-cm14);
    const double pr7_2 = x[3] * (-cm17);
    const double pr7_3 = x[4] * (-cm20);
    const double pr7_4 = x[5] * (-cm22);
    const double pr7_5 = x[6] * (-cm23);
    const double b0 = (((((pr0_0 + pr0_1) + pr0_2) + pr0_3) + pr0_4) + pr0_5) * twelth;
    bmat[(size_t)2 * ne + e] = b0;
    Sz = w[0] * b0;
    const double b1 = (((((pr1_0 + pr1_1) + pr1_2) + pr1_3) + pr1_4) + pr1_5) * twelth;
    bmat[(size_t)5 * ne + e] = b1;
    Sz = Sz + w[1] * b1;
    const double b2 = (((((pr2_0 + pr2_1) + pr2_2) + pr2_3) + pr2_4) + pr2_5) * twelth;
    bmat[(size_t)8 * ne + e] = b2;
    Sz = Sz + w[2] * b2;
    const double b3 = (((((pr3_0 + pr3_1) + pr3_2) + pr3_3) + pr3_4) + pr3_5) * twelth;
    bmat[(size_t)11 * ne + e] = b3;
    Sz = Sz + w[3] * b3;
    const double b4 = (((((pr4_0 + pr4_1) + pr4_2) + pr4_3) + pr4_4) + pr4_5) * twelth;
    bmat[(size_t)14 * ne + e] = b4;
    Sz = Sz + w[4] * b4;
    const double b5 = (((((pr5_0 + pr5_1) + pr5_2) + pr5_3) + pr5_4) + pr5_5) * twelth;
    bmat[(size_t)17 * ne + e] = b5;
    Sz = Sz + w[5] * b5;
    const double b6 = (((((pr6_0 + pr6_1) + pr6_2) + pr6_3) + pr6_4) + pr6_5) * twelth;
    bmat[(size_t)20 * ne + e] = b6;
    Sz = Sz + w[6] * b6;
    const double b7 = (((((pr7_0 + pr7_1) + pr7_2) + pr7_3) + pr7_4) + pr7_5) * twelth;
    bmat[(size_t)23 * ne + e] = b7;
    Sz = Sz + w[7] * b7;
  }
}

// The exact hex volume alone (geometry.cpp:271-310), the same operations in the
// same order as hex_geometry's volume.
__device__ __forceinline__ double hex_volume(const double* __restrict__ x, const double* __restrict__ y,
    const double* __restrict__ z) {
  const double twelth = 1. / 12.;
  const double cm0 = (((-z[2] - z[3]) + z[4]) + z[5]);
  const double cm1 = (z[1] - z[3]);
  const double cm2 = (((z[1] + z[2]) - z[4]) - z[7]);
  const double cm3 = (((-z[1] + z[3]) - z[5]) + z[7]);
  const double cm4 = (-z[1] + z[4]);
  const double cm5 = (z[3] - z[4]);
  const double cm6 = (((-z[0] - z[3]) + z[5]) + z[6]);
  const double cm7 = (-z[0] + z[2]);
  const double cm8 = (z[0] - z[5]);
  const double cm9 = (((z[0] - z[2]) + z[4]) - z[6]);
  const double cm10 = (-z[2] + z[5]);
  const double cm11 = (((-z[0] - z[1]) + z[6]) + z[7]);
  const double cm12 = (z[1] - z[6]);
  const double cm13 = (((z[1] - z[3]) + z[5]) - z[7]);
  const double cm14 = (-z[3] + z[6]);
  const double cm15 = (-z[0] + z[7]);
  const double cm16 = (z[2] - z[7]);
  const double cm17 = (((-z[0] + z[2]) - z[4]) + z[6]);
  const double cm18 = (((-z[0] - z[1]) + z[6]) + z[7]);
  const double cm19 = (-z[5] + z[7]);
  const double cm20 = (((z[0] + z[3]) - z[5]) - z[6]);
  const double cm21 = (((-z[1] - z[2]) + z[4]) + z[7]);
  const double cm22 = (z[4] - z[6]);
  const double cm23 = (((-z[2] - z[3]) + z[4]) + z[5]);
  const double pr0_0 = y[1] * cm0;
  const double pr0_1 = y[2] * cm1;
  const double pr0_2 = y[3] * cm2;
  const double pr0_3 = y[4] * cm3;
  const double pr0_4 = y[5] * cm4;
  const double pr0_5 = y[7] * cm5;
  const double pr1_0 = y[0] * (-cm0);
  const double pr1_1 = y[2] * cm6;
  const double pr1_2 = y[3] * cm7;
  const double pr1_3 = y[4] * cm8;
  const double pr1_4 = y[5] * cm9;
  const double pr1_5 = y[6] * cm10;
  const double pr2_0 = y[0] * (-cm1);
  const double pr2_1 = y[1] * (-cm6);
  const double pr2_2 = y[3] * cm11;
  const double pr2_3 = y[5] * cm12;
  const double pr2_4 = y[6] * cm13;
  const double pr2_5 = y[7] * cm14;
  const double pr3_0 = y[0] * (-cm2);
  const double pr3_1 = y[1] * (-cm7);
  const double pr3_2 = y[2] * (-cm11);
  const double pr3_3 = y[4] * cm15;
  const double pr3_4 = y[6] * cm16;
  const double pr3_5 = y[7] * cm17;
  const double pr4_0 = y[0] * (-cm3);
  const double pr4_1 = y[1] * (-cm8);
  const double pr4_2 = y[3] * (-cm15);
  const double pr4_3 = y[5] * cm18;
  const double pr4_4 = y[6] * cm19;
  const double pr4_5 = y[7] * cm20;
  const double pr5_0 = y[0] * (-cm4);
  const double pr5_1 = y[1] * (-cm9);
  const double pr5_2 = y[2] * (-cm12);
  const double pr5_3 = y[4] * (-cm18);
  const double pr5_4 = y[6] * cm21;
  const double pr5_5 = y[7] * cm22;
  const double pr6_0 = y[1] * (-cm10);
  const double pr6_1 = y[2] * (-cm13);
  const double pr6_2 = y[3] * (-cm16);
  const double pr6_3 = y[4] * (-cm19);
  const double pr6_4 = y[5] * (-cm21);
  const double pr6_5 = y[7] * cm23;
  const double pr7_0 = y[0] * (-cm5);
  const double pr7_1 = y[2] * (-cm14);
  const double pr7_2 = y[3] * (-cm17);
  const double pr7_3 = y[4] * (-cm20);
  const double pr7_4 = y[5] * (-cm22);
  const double pr7_5 = y[6] * (-cm23);
  const double vi0 = x[1] * (((((pr1_2 + pr1_3) + pr1_0) + pr1_5) + pr1_4) + pr1_1);
  const double vi1 = x[7] * (((((pr7_0 + pr7_5) + pr7_1) + pr7_2) + pr7_4) + pr7_3);
  const double vi2 = x[3] * (((((pr3_1 + pr3_5) + pr3_4) + pr3_2) + pr3_3) + pr3_0);
  const double vi3 = x[5] * (((((pr5_0 + pr5_5) + pr5_2) + pr5_1) + pr5_3) + pr5_4);
  const double vi4 = x[6] * (((((pr6_0 + pr6_5) + pr6_4) + pr6_3) + pr6_2) + pr6_1);
  const double vi5 = x[0] * (((((pr0_1 + pr0_5) + pr0_4) + pr0_0) + pr0_2) + pr0_3);
  const double vi6 = x[2] * (((((pr2_0 + pr2_3) + pr2_1) + pr2_5) + pr2_4) + pr2_2);
  const double vi7 = x[4] * (((((pr4_1 + pr4_5) + pr4_2) + pr4_0) + pr4_4) + pr4_3);
  return (((((((vi0 + vi1) + vi2) + vi3) + vi4) + vi5) + vi6) + vi7) * twelth;
}

// Reverse mode of the corner normals: given Bbar[lid*3+dim] (the adjoint of
// B(lid, dim)), accumulate the coordinate adjoints xbar, ybar, zbar[8].  B is
// bilinear, B(p,c) = sum_t O[j_t] comb_t(I) / 12, and each unordered pair (p, j)
// enters B(p) as O[j] cm and B(j) as -O[p] cm with one shared combo cm, so
//   Obar[j] += g_p cm,  Obar[p] -= g_j cm,  Ibar[terms of cm] +-= g_p O[j] - g_j O[p]
// with g = Bbar / 12 (multiply-adds fused: the adjoint has no parity target).
__device__ __forceinline__ void hex_bmatrix_adjoint(const double* __restrict__ x, const double* __restrict__ y,
    const double* __restrict__ z, const double* __restrict__ Bbar, double* __restrict__ xbar,
    double* __restrict__ ybar, double* __restrict__ zbar) {
  const double twelth = 1. / 12.;
  {  // component 0: O = y, I = z
    const double g0 = Bbar[0] * twelth;
    const double g1 = Bbar[3] * twelth;
    const double g2 = Bbar[6] * twelth;
    const double g3 = Bbar[9] * twelth;
    const double g4 = Bbar[12] * twelth;
    const double g5 = Bbar[15] * twelth;
    const double g6 = Bbar[18] * twelth;
    const double g7 = Bbar[21] * twelth;
    {  // pair (0,1)
      const double cm = (((-z[2] - z[3]) + z[4]) + z[5]);
      ybar[1] = fma(g0, cm, ybar[1]);
      ybar[0] = fma(-g1, cm, ybar[0]);
      const double wk = fma(g0, y[1], -(g1 * y[0]));
      zbar[2] -= wk;
      zbar[3] -= wk;
      zbar[4] += wk;
      zbar[5] += wk;
    }
    {  // pair (0,2)
      const double cm = (z[1] - z[3]);
      ybar[2] = fma(g0, cm, ybar[2]);
      ybar[0] = fma(-g2, cm, ybar[0]);
      const double wk = fma(g0, y[2], -(g2 * y[0]));
      zbar[1] += wk;
      zbar[3] -= wk;
    }
    {  // pair (0,3)
      const double cm = (((z[1] + z[2]) - z[4]) - z[7]);
      ybar[3] = fma(g0, cm, ybar[3]);
      ybar[0] = fma(-g3, cm, ybar[0]);
      const double wk = fma(g0, y[3], -(g3 * y[0]));
      zbar[1] += wk;
      zbar[2] += wk;
      zbar[4] -= wk;
      zbar[7] -= wk;
    }
    {  // pair (0,4)
      const double cm = (((-z[1] + z[3]) - z[5]) + z[7]);
      ybar[4] = fma(g0, cm, ybar[4]);
      ybar[0] = fma(-g4, cm, ybar[0]);
      const double wk = fma(g0, y[4], -(g4 * y[0]));
      zbar[1] -= wk;
      zbar[3] += wk;
      zbar[5] -= wk;
      zbar[7] += wk;
    }
    {  // pair (0,5)
      const double cm = (-z[1] + z[4]);
      ybar[5] = fma(g0, cm, ybar[5]);
      ybar[0] = fma(-g5, cm, ybar[0]);
      const double wk = fma(g0, y[5], -(g5 * y[0]));
      zbar[1] -= wk;
      zbar[4] += wk;
    }
    {  // pair (0,7)
      const double cm = (z[3] - z[4]);
      ybar[7] = fma(g0, cm, ybar[7]);
      ybar[0] = fma(-g7, cm, ybar[0]);
      const double wk = fma(g0, y[7], -(g7 * y[0]));
      zbar[3] += wk;
      zbar[4] -= wk;
    }
    {  // pair (1,2)
      const double cm = (((-z[0] - z[3]) + z[5]) + z[6]);
      ybar[2] = fma(g1, cm, ybar[2]);
      ybar[1] = fma(-g2, cm, ybar[1]);
      const double wk = fma(g1, y[2], -(g2 * y[1]));
      zbar[0] -= wk;
      zbar[3] -= wk;
      zbar[5] += wk;
      zbar[6] += wk;
    }
    {  // pair (1,3)
      const double cm = (-z[0] + z[2]);
      ybar[3] = fma(g1, cm, ybar[3]);
      ybar[1] = fma(-g3, cm, ybar[1]);
      const double wk = fma(g1, y[3], -(g3 * y[1]));
      zbar[0] -= wk;
      zbar[2] += wk;
    }
    {  // pair (1,4)
      const double cm = (z[0] - z[5]);
      ybar[4] = fma(g1, cm, ybar[4]);
      ybar[1] = fma(-g4, cm, ybar[1]);
      const double wk = fma(g1, y[4], -(g4 * y[1]));
      zbar[0] += wk;
      zbar[5] -= wk;
    }
    {  // pair (1,5)
      const double cm = (((z[0] - z[2]) + z[4]) - z[6]);
      ybar[5] = fma(g1, cm, ybar[5]);
      ybar[1] = fma(-g5, cm, ybar[1]);
      const double wk = fma(g1, y[5], -(g5 * y[1]));
      zbar[0] += wk;
      zbar[2] -= wk;
      zbar[4] += wk;
      zbar[6] -= wk;
    }
    {  // pair (1,6)
      const double cm = (-z[2] + z[5]);
      ybar[6] = fma(g1, cm, ybar[6]);
      ybar[1] = fma(-g6, cm, ybar[1]);
      const double wk = fma(g1, y[6], -(g6 * y[1]));
      zbar[2] -= wk;
      zbar[5] += wk;
    }
    {  // pair (2,3)
      const double cm = (((-z[0] - z[1]) + z[6]) + z[7]);
      ybar[3] = fma(g2, cm, ybar[3]);
      ybar[2] = fma(-g3, cm, ybar[2]);
      const double wk = fma(g2, y[3], -(g3 * y[2]));
      zbar[0] -= wk;
      zbar[1] -= wk;
      zbar[6] += wk;
      zbar[7] += wk;
    }
    {  // pair (2,5)
      const double cm = (z[1] - z[6]);
      ybar[5] = fma(g2, cm, ybar[5]);
      ybar[2] = fma(-g5, cm, ybar[2]);
      const double wk = fma(g2, y[5], -(g5 * y[2]));
      zbar[1] += wk;
      zbar[6] -= wk;
    }
    {  // pair (2,6)
      const double cm = (((z[1] - z[3]) + z[5]) - z[7]);
      ybar[6] = fma(g2, cm, ybar[6]);
      ybar[2] = fma(-g6, cm, ybar[2]);
      const double wk = fma(g2, y[6], -(g6 * y[2]));
      zbar[1] += wk;
      zbar[3] -= wk;
      zbar[5] += wk;
      zbar[7] -= wk;
    }
    {  // pair (2,7)
      const double cm = (-z[3] + z[6]);
      ybar[7] = fma(g2, cm, ybar[7]);
      ybar[2] = fma(-g7, cm, ybar[2]);
      const double wk = fma(g2, y[7], -(g7 * y[2]));
      zbar[3] -= wk;
      zbar[6] += wk;
    }
    {  // pair (3,4)
      const double cm = (-z[0] + z[7]);
      ybar[4] = fma(g3, cm, ybar[4]);
      ybar[3] = fma(-g4, cm, ybar[3]);
      const double wk = fma(g3, y[4], -(g4 * y[3]));
      zbar[0] -= wk;
      zbar[7] += wk;
    }
    {  // pair (3,6)
      const double cm = (z[2] - z[7]);
      ybar[6] = fma(g3, cm, ybar[6]);
      ybar[3] = fma(-g6, cm, ybar[3]);
      const double wk = fma(g3, y[6], -(g6 * y[3]));
      zbar[2] += wk;
      zbar[7] -= wk;
    }
    {  // pair (3,7)
      const double cm = (((-z[0] + z[2]) - z[4]) + z[6]);
      ybar[7] = fma(g3, cm, ybar[7]);
      ybar[3] = fma(-g7, cm, ybar[3]);
      const double wk = fma(g3, y[7], -(g7 * y[3]));
      zbar[0] -= wk;
      zbar[2] += wk;
      zbar[4] -= wk;
      zbar[6] += wk;
    }
    {  // pair (4,5)
      const double cm = (((-z[0] - z[1]) + z[6]) + z[7]);
      ybar[5] = fma(g4, cm, ybar[5]);
      ybar[4] = fma(-g5, cm, ybar[4]);
      const double wk = fma(g4, y[5], -(g5 * y[4]));
      zbar[0] -= wk;
      zbar[1] -= wk;
      zbar[6] += wk;
      zbar[7] += wk;
    }
    {  // pair (4,6)
      const double cm = (-z[5] + z[7]);
      ybar[6] = fma(g4, cm, ybar[6]);
      ybar[4] = fma(-g6, cm, ybar[4]);
      const double wk = fma(g4, y[6], -(g6 * y[4]));
      zbar[5] -= wk;
      zbar[7] += wk;
    }
    {  // pair (4,7)
      const double cm = (((z[0] + z[3]) - z[5]) - z[6]);
      ybar[7] = fma(g4, cm, ybar[7]);
      ybar[4] = fma(-g7, cm, ybar[4]);
      const double wk = fma(g4, y[7], -(g7 * y[4]));
      zbar[0] += wk;
      zbar[3] += wk;
      zbar[5] -= wk;
      zbar[6] -= wk;
    }
    {  // pair (5,6)
      const double cm = (((-z[1] - z[2]) + z[4]) + z[7]);
      ybar[6] = fma(g5, cm, ybar[6]);
      ybar[5] = fma(-g6, cm, ybar[5]);
      const double wk = fma(g5, y[6], -(g6 * y[5]));
      zbar[1] -= wk;
      zbar[2] -= wk;
      zbar[4] += wk;
      zbar[7] += wk;
    }
    {  // pair (5,7)
      const double cm = (z[4] - z[6]);
      ybar[7] = fma(g5, cm, ybar[7]);
      ybar[5] = fma(-g7, cm, ybar[5]);
      const double wk = fma(g5, y[7], -(g7 * y[5]));
      zbar[4] += wk;
      zbar[6] -= wk;
    }
    {  // pair (6,7)
      const double cm = (((-z[2] - z[3]) + z[4]) + z[5]);
      ybar[7] = fma(g6, cm, ybar[7]);
      ybar[6] = fma(-g7, cm, ybar[6]);
      const double wk = fma(g6, y[7], -(g7 * y[6]));
      zbar[2] -= wk;
      zbar[3] -= wk;
      zbar[4] += wk;
      zbar[5] += wk;
    }
  }
  {  // component 1: O = z, I = x
    const double g0 = Bbar[1] * twelth;
    const double g1 = Bbar[4] * twelth;
    const double g2 = Bbar[7] * twelth;
    const double g3 = Bbar[10] * twelth;
    const double g4 = Bbar[13] * twelth;
    const double g5 = Bbar[16] * twelth;
    const double g6 = Bbar[19] * twelth;
    const double g7 = Bbar[22] * twelth;
    {  // pair (0,1)
      const double cm = (((-x[2] - x[3]) + x[4]) + x[5]);
      zbar[1] = fma(g0, cm, zbar[1]);
      zbar[0] = fma(-g1, cm, zbar[0]);
      const double wk = fma(g0, z[1], -(g1 * z[0]));
      xbar[2] -= wk;
      xbar[3] -= wk;
      xbar[4] += wk;
      xbar[5] += wk;
    }
    {  // pair (0,2)
      const double cm = (x[1] - x[3]);
      zbar[2] = fma(g0, cm, zbar[2]);
      zbar[0] = fma(-g2, cm, zbar[0]);
      const double wk = fma(g0, z[2], -(g2 * z[0]));
      xbar[1] += wk;
      xbar[3] -= wk;
    }
    {  // pair (0,3)
      const double cm = (((x[1] + x[2]) - x[4]) - x[7]);
      zbar[3] = fma(g0, cm, zbar[3]);
      zbar[0] = fma(-g3, cm, zbar[0]);
      const double wk = fma(g0, z[3], -(g3 * z[0]));
      xbar[1] += wk;
      xbar[2] += wk;
      xbar[4] -= wk;
      xbar[7] -= wk;
    }
    {  // pair (0,4)
      const double cm = (((-x[1] + x[3]) - x[5]) + x[7]);
      zbar[4] = fma(g0, cm, zbar[4]);
      zbar[0] = fma(-g4, cm, zbar[0]);
      const double wk = fma(g0, z[4], -(g4 * z[0]));
      xbar[1] -= wk;
      xbar[3] += wk;
      xbar[5] -= wk;
      xbar[7] += wk;
    }
    {  // pair (0,5)
      const double cm = (-x[1] + x[4]);
      zbar[5] = fma(g0, cm, zbar[5]);
      zbar[0] = fma(-g5, cm, zbar[0]);
      const double wk = fma(g0, z[5], -(g5 * z[0]));
      xbar[1] -= wk;
      xbar[4] += wk;
    }
    {  // pair (0,7)
      const double cm = (x[3] - x[4]);
      zbar[7] = fma(g0, cm, zbar[7]);
      zbar[0] = fma(-g7, cm, zbar[0]);
      const double wk = fma(g0, z[7], -(g7 * z[0]));
      xbar[3] += wk;
      xbar[4] -= wk;
    }
    {  // pair (1,2)
      const double cm = (((-x[0] - x[3]) + x[5]) + x[6]);
      zbar[2] = fma(g1, cm, zbar[2]);
      zbar[1] = fma(-g2, cm, zbar[1]);
      const double wk = fma(g1, z[2], -(g2 * z[1]));
      xbar[0] -= wk;
      xbar[3] -= wk;
      xbar[5] += wk;
      xbar[6] += wk;
    }
    {  // pair (1,3)
      const double cm = (-x[0] + x[2]);
      zbar[3] = fma(g1, cm, zbar[3]);
      zbar[1] = fma(-g3, cm, zbar[1]);
      const double wk = fma(g1, z[3], -(g3 * z[1]));
      xbar[0] -= wk;
      xbar[2] += wk;
    }
    {  // pair (1,4)
      const double cm = (x[0] - x[5]);
      zbar[4] = fma(g1, cm, zbar[4]);
      zbar[1] = fma(-g4, cm, zbar[1]);
      const double wk = fma(g1, z[4], -(g4 * z[1]));
      xbar[0] += wk;
      xbar[5] -= wk;
    }
    {  // pair (1,5)
      const double cm = (((x[0] - x[2]) + x[4]) - x[6]);
      zbar[5] = fma(g1, cm, zbar[5]);
      zbar[1] = fma(-g5, cm, zbar[1]);
      const double wk = fma(g1, z[5], -(g5 * z[1]));
      xbar[0] += wk;
      xbar[2] -= wk;
      xbar[4] += wk;
      xbar[6] -= wk;
    }
    {  // pair (1,6)
      const double cm = (-x[2] + x[5]);
      zbar[6] = fma(g1, cm, zbar[6]);
      zbar[1] = fma(-g6, cm, zbar[1]);
      const double wk = fma(g1, z[6], -(g6 * z[1]));
      xbar[2] -= wk;
      xbar[5] += wk;
    }
    {  // pair (2,3)
      const double cm = (((-x[0] - x[1]) + x[6]) + x[7]);
      zbar[3] = fma(g2, cm, zbar[3]);
      zbar[2] = fma(-g3, cm, zbar[2]);
      const double wk = fma(g2, z[3], -(g3 * z[2]));
      xbar[0] -= wk;
      xbar[1] -= wk;
      xbar[6] += wk;
      xbar[7] += wk;
    }
    {  // pair (2,5)
      const double cm = (x[1] - x[6]);
      zbar[5] = fma(g2, cm, zbar[5]);
      zbar[2] = fma(-g5, cm, zbar[2]);
      const double wk = fma(g2, z[5], -(g5 * z[2]));
      xbar[1] += wk;
      xbar[6] -= wk;
    }
    {  // pair (2,6)
      const double cm = (((x[1] - x[3]) + x[5]) - x[7]);
      zbar[6] = fma(g2, cm, zbar[6]);
      zbar[2] = fma(-g6, cm, zbar[2]);
      const double wk = fma(g2, z[6], -(g6 * z[2]));
      xbar[1] += wk;
      xbar[3] -= wk;
      xbar[5] += wk;
      xbar[7] -= wk;
    }
    {  // pair (2,7)
      const double cm = (-x[3] + x[6]);
      zbar[7] = fma(g2, cm, zbar[7]);
      zbar[2] = fma(-g7, cm, zbar[2]);
      const double wk = fma(g2, z[7], -(g7 * z[2]));
      xbar[3] -= wk;
      xbar[6] += wk;
    }
    {  // pair (3,4)
      const double cm = (-x[0] + x[7]);
      zbar[4] = fma(g3, cm, zbar[4]);
      zbar[3] = fma(-g4, cm, zbar[3]);
      const double wk = fma(g3, z[4], -(g4 * z[3]));
      xbar[0] -= wk;
      xbar[7] += wk;
    }
    {  // pair (3,6)
      const double cm = (x[2] - x[7]);
      zbar[6] = fma(g3, cm, zbar[6]);
      zbar[3] = fma(-g6, cm, zbar[3]);
      const double wk = fma(g3, z[6], -(g6 * z[3]));
      xbar[2] += wk;
      xbar[7] -= wk;
    }
    {  // pair (3,7)
      const double cm = (((-x[0] + x[2]) - x[4]) + x[6]);
      zbar[7] = fma(g3, cm, zbar[7]);
      zbar[3] = fma(-g7, cm, zbar[3]);
      const double wk = fma(g3, z[7], -(g7 * z[3]));
      xbar[0] -= wk;
      xbar[2] += wk;
      xbar[4] -= wk;
      xbar[6] += wk;
    }
    {  // pair (4,5)
      const double cm = (((-x[0] - x[1]) + x[6]) + x[7]);
      zbar[5] = fma(g4, cm, zbar[5]);
      zbar[4] = fma(-g5, cm, zbar[4]);
      const double wk = fma(g4, z[5], -(g5 * z[4]));
      xbar[0] -= wk;
      xbar[1] -= wk;
      xbar[6] += wk;
      xbar[7] += wk;
    }
    {  // pair (4,6)
      const double cm = (-x[5] + x[7]);
      zbar[6] = fma(g4, cm, zbar[6]);
      zbar[4] = fma(-g6, cm, zbar[4]);
      const double wk = fma(g4, z[6], -(g6 * z[4]));
      xbar[5] -= wk;
      xbar[7] += wk;
    }
    {  // pair (4,7)
      const double cm = (((x[0] + x[3]) - x[5]) - x[6]);
      zbar[7] = fma(g4, cm, zbar[7]);
      zbar[4] = fma(-g7, cm, zbar[4]);
      const double wk = fma(g4, z[7], -(g7 * z[4]));
      xbar[0] += wk;
      xbar[3] += wk;
      xbar[5] -= wk;
      xbar[6] -= wk;
    }
    {  // pair (5,6)
      const double cm = (((-x[1] - x[2]) + x[4]) + x[7]);
      zbar[6] = fma(g5, cm, zbar[6]);
      zbar[5] = fma(-g6, cm, zbar[5]);
      const double wk = fma(g5, z[6], -(g6 * z[5]));
      xbar[1] -= wk;
      xbar[2] -= wk;
      xbar[4] += wk;
      xbar[7] += wk;
    }
    {  // pair (5,7)
      const double cm = (x[4] - x[6]);
      zbar[7] = fma(g5, cm, zbar[7]);
      zbar[5] = fma(-g7, cm, zbar[5]);
      const double wk = fma(g5, z[7], -(g7 * z[5]));
      xbar[4] += wk;
      xbar[6] -= wk;
    }
    {  // pair (6,7)
      const double cm = (((-x[2] - x[3]) + x[4]) + x[5]);
      zbar[7] = fma(g6, cm, zbar[7]);
      zbar[6] = fma(-g7, cm, zbar[6]);
      const double wk = fma(g6, z[7], -(g7 * z[6]));
      xbar[2] -= wk;
      xbar[3] -= wk;
      xbar[4] += wk;
      xbar[5] += wk;
    }
  }
  {  // component 2: O = x, I = y
    const double g0 = Bbar[2] * twelth;
    const double g1 = Bbar[5] * twelth;
    const double g2 = Bbar[8] * twelth;
    const double g3 = Bbar[11] * twelth;
    const double g4 = Bbar[14] * twelth;
    const double g5 = Bbar[17] * twelth;
    const double g6 = Bbar[20] * twelth;
    const double g7 = Bbar[23] * twelth;
    {  // pair (0,1)
      const double cm = (((-y[2] - y[3]) + y[4]) + y[5]);
      xbar[1] = fma(g0, cm, xbar[1]);
      xbar[0] = fma(-g1, cm, xbar[0]);
      const double wk = fma(g0, x[1], -(g1 * x[0]));
      ybar[2] -= wk;
      ybar[3] -= wk;
      ybar[4] += wk;
      ybar[5] += wk;
    }
    {  // pair (0,2)
      const double cm = (y[1] - y[3]);
      xbar[2] = fma(g0, cm, xbar[2]);
      xbar[0] = fma(-g2, cm, xbar[0]);
      const double wk = fma(g0, x[2], -(g2 * x[0]));
      ybar[1] += wk;
      ybar[3] -= wk;
    }
    {  // pair (0,3)
      const double cm = (((y[1] + y[2]) - y[4]) - y[7]);
      xbar[3] = fma(g0, cm, xbar[3]);
      xbar[0] = fma(-g3, cm, xbar[0]);
      const double wk = fma(g0, x[3], -(g3 * x[0]));
      ybar[1] += wk;
      ybar[2] += wk;
      ybar[4] -= wk;
      ybar[7] -= wk;
    }
    {  // pair (0,4)
      const double cm = (((-y[1] + y[3]) - y[5]) + y[7]);
      xbar[4] = fma(g0, cm, xbar[4]);
      xbar[0] = fma(-g4, cm, xbar[0]);
      const double wk = fma(g0, x[4], -(g4 * x[0]));
      ybar[1] -= wk;
      ybar[3] += wk;
      ybar[5] -= wk;
      ybar[7] += wk;
    }
    {  // pair (0,5)
      const double cm = (-y[1] + y[4]);
      xbar[5] = fma(g0, cm, xbar[5]);
      xbar[0] = fma(-g5, cm, xbar[0]);
      const double wk = fma(g0, x[5], -(g5 * x[0]));
      ybar[1] -= wk;
      ybar[4] += wk;
    }
    {  // pair (0,7)
      const double cm = (y[3] - y[4]);
      xbar[7] = fma(g0, cm, xbar[7]);
      xbar[0] = fma(-g7, cm, xbar[0]);
      const double wk = fma(g0, x[7], -(g7 * x[0]));
      ybar[3] += wk;
      ybar[4] -= wk;
    }
    {  // pair (1,2)
      const double cm = (((-y[0] - y[3]) + y[5]) + y[6]);
      xbar[2] = fma(g1, cm, xbar[2]);
      xbar[1] = fma(-g2, cm, xbar[1]);
      const double wk = fma(g1, x[2], -(g2 * x[1]));
      ybar[0] -= wk;
      ybar[3] -= wk;
      ybar[5] += wk;
      ybar[6] += wk;
    }
    {  // pair (1,3)
      const double cm = (-y[0] + y[2]);
      xbar[3] = fma(g1, cm, xbar[3]);
      xbar[1] = fma(-g3, cm, xbar[1]);
      const double wk = fma(g1, x[3], -(g3 * x[1]));
      ybar[0] -= wk;
      ybar[2] += wk;
    }
    {  // pair (1,4)
      const double cm = (y[0] - y[5]);
      xbar[4] = fma(g1, cm, xbar[4]);
      xbar[1] = fma(-g4, cm, xbar[1]);
      const double wk = fma(g1, x[4], -(g4 * x[1]));
      ybar[0] += wk;
      ybar[5] -= wk;
    }
    {  // pair (1,5)
      const double cm = (((y[0] - y[2]) + y[4]) - y[6]);
      xbar[5] = fma(g1, cm, xbar[5]);
      xbar[1] = fma(-g5, cm, xbar[1]);
      const double wk = fma(g1, x[5], -(g5 * x[1]));
      ybar[0] += wk;
      ybar[2] -= wk;
      ybar[4] += wk;
      ybar[6] -= wk;
    }
    {  // pair (1,6)
      const double cm = (-y[2] + y[5]);
      xbar[6] = fma(g1, cm, xbar[6]);
      xbar[1] = fma(-g6, cm, xbar[1]);
      const double wk = fma(g1, x[6], -(g6 * x[1]));
      ybar[2] -= wk;
      ybar[5] += wk;
    }
    {  // pair (2,3)
      const double cm = (((-y[0] - y[1]) + y[6]) + y[7]);
      xbar[3] = fma(g2, cm, xbar[3]);
      xbar[2] = fma(-g3, cm, xbar[2]);
      const double wk = fma(g2, x[3], -(g3 * x[2]));
      ybar[0] -= wk;
      ybar[1] -= wk;
      ybar[6] += wk;
      ybar[7] += wk;
    }
    {  // pair (2,5)
      const double cm = (y[1] - y[6]);
      xbar[5] = fma(g2, cm, xbar[5]);
      xbar[2] = fma(-g5, cm, xbar[2]);
      const double wk = fma(g2, x[5], -(g5 * x[2]));
      ybar[1] += wk;
      ybar[6] -= wk;
    }
    {  // pair (2,6)
      const double cm = (((y[1] - y[3]) + y[5]) - y[7]);
      xbar[6] = fma(g2, cm, xbar[6]);
      xbar[2] = fma(-g6, cm, xbar[2]);
      const double wk = fma(g2, x[6], -(g6 * x[2]));
      ybar[1] += wk;
      ybar[3] -= wk;
      ybar[5] += wk;
      ybar[7] -= wk;
    }
    {  // pair (2,7)
      const double cm = (-y[3] + y[6]);
      xbar[7] = fma(g2, cm, xbar[7]);
      xbar[2] = fma(-g7, cm, xbar[2]);
      const double wk = fma(g2, x[7], -(g7 * x[2]));
      ybar[3] -= wk;
      ybar[6] += wk;
    }
    {  // pair (3,4)
      const double cm = (-y[0] + y[7]);
      xbar[4] = fma(g3, cm, xbar[4]);
      xbar[3] = fma(-g4, cm, xbar[3]);
      const double wk = fma(g3, x[4], -(g4 * x[3]));
      ybar[0] -= wk;
      ybar[7] += wk;
    }
    {  // pair (3,6)
      const double cm = (y[2] - y[7]);
      xbar[6] = fma(g3, cm, xbar[6]);
      xbar[3] = fma(-g6, cm, xbar[3]);
      const double wk = fma(g3, x[6], -(g6 * x[3]));
      ybar[2] += wk;
      ybar[7] -= wk;
    }
    {  // pair (3,7)
      const double cm = (((-y[0] + y[2]) - y[4]) + y[6]);
      xbar[7] = fma(g3, cm, xbar[7]);
      xbar[3] = fma(-g7, cm, xbar[3]);
      const double wk = fma(g3, x[7], -(g7 * x[3]));
      ybar[0] -= wk;
      ybar[2] += wk;
      ybar[4] -= wk;
      ybar[6] += wk;
    }
    {  // pair (4,5)
      const double cm = (((-y[0] - y[1]) + y[6]) + y[7]);
      xbar[5] = fma(g4, cm, xbar[5]);
      xbar[4] = fma(-g5, cm, xbar[4]);
      const double wk = fma(g4, x[5], -(g5 * x[4]));
      ybar[0] -= wk;
      ybar[1] -= wk;
      ybar[6] += wk;
      ybar[7] += wk;
    }
    {  // pair (4,6)
      const double cm = (-y[5] + y[7]);
      xbar[6] = fma(g4, cm, xbar[6]);
      xbar[4] = fma(-g6, cm, xbar[4]);
      const double wk = fma(g4, x[6], -(g6 * x[4]));
      ybar[5] -= wk;
      ybar[7] += wk;
    }
    {  // pair (4,7)
      const double cm = (((y[0] + y[3]) - y[5]) - y[6]);
      xbar[7] = fma(g4, cm, xbar[7]);
      xbar[4] = fma(-g7, cm, xbar[4]);
      const double wk = fma(g4, x[7], -(g7 * x[4]));
      ybar[0] += wk;
      ybar[3] += wk;
      ybar[5] -= wk;
      ybar[6] -= wk;
    }
    {  // pair (5,6)
      const double cm = (((-y[1] - y[2]) + y[4]) + y[7]);
      xbar[6] = fma(g5, cm, xbar[6]);
      xbar[5] = fma(-g6, cm, xbar[5]);
      const double wk = fma(g5, x[6], -(g6 * x[5]));
      ybar[1] -= wk;
      ybar[2] -= wk;
      ybar[4] += wk;
      ybar[7] += wk;
    }
    {  // pair (5,7)
      const double cm = (y[4] - y[6]);
      xbar[7] = fma(g5, cm, xbar[7]);
      xbar[5] = fma(-g7, cm, xbar[5]);
      const double wk = fma(g5, x[7], -(g7 * x[5]));
      ybar[4] += wk;
      ybar[6] -= wk;
    }
    {  // pair (6,7)
      const double cm = (((-y[2] - y[3]) + y[4]) + y[5]);
      xbar[7] = fma(g6, cm, xbar[7]);
      xbar[6] = fma(-g7, cm, xbar[6]);
      const double wk = fma(g6, x[7], -(g7 * x[6]));
      ybar[2] -= wk;
      ybar[3] -= wk;
      ybar[4] += wk;
      ybar[5] += wk;
    }
  }
}
