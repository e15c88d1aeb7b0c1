// GENERATED by gen_hex_geometry.py from sgh_hex.h -- do not edit.
// Straight-line hex geometry; see the generator's docstring for the exactness argument.
#pragma once

// In: x,y,z,u,v,w[8] (node lids 0..7).  Out: vol; bmat rows lid*3+dim at
// bmat[row*ne + e]; Sx,Sy,Sz = sum_p u_p B(p,0), v_p B(p,1), w_p B(p,2) (p order);
// with CFL, d2min = min over the 28 node pairs of the squared distance.
template <bool CFL>
__device__ __forceinline__ void hex_geometry(const double* __restrict__ x, const double* __restrict__ y,
    const double* __restrict__ z, const double* __restrict__ u, const double* __restrict__ v,
    const double* __restrict__ w, double* __restrict__ bmat, int ne, int e, double& vol,
    double& Sx, double& Sy, double& Sz, double& d2min) {
  const double twelth = 1. / 12.;
  double dz_0_2, dz_0_5, dz_0_7, dz_1_3, dz_1_4, dz_1_6, dz_2_5, dz_2_7, dz_3_4, dz_3_6, dz_4_6, dz_5_7, dx_0_2, dx_0_5, dx_0_7, dx_1_3, dx_1_4, dx_1_6, dx_2_5, dx_2_7, dx_3_4, dx_3_6, dx_4_6, dx_5_7, dy_0_2, dy_0_5, dy_0_7, dy_1_3, dy_1_4, dy_1_6, dy_2_5, dy_2_7, dy_3_4, dy_3_6, dy_4_6, dy_5_7;
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
    vol = (((((((vi0 + vi1) + vi2) + vi3) + vi4) + vi5) + vi6) + vi7) * twelth;
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
    const double fd_z_0_2 = cm7;
    const double fd_z_0_5 = cm8;
    const double fd_z_0_7 = cm15;
    const double fd_z_1_3 = cm1;
    const double fd_z_1_4 = cm4;
    const double fd_z_1_6 = cm12;
    const double fd_z_2_5 = cm10;
    const double fd_z_2_7 = cm16;
    const double fd_z_3_4 = cm5;
    const double fd_z_3_6 = cm14;
    const double fd_z_4_6 = cm22;
    const double fd_z_5_7 = cm19;
    dz_0_2 = fd_z_0_2; dz_0_5 = fd_z_0_5; dz_0_7 = fd_z_0_7; dz_1_3 = fd_z_1_3; dz_1_4 = fd_z_1_4; dz_1_6 = fd_z_1_6; dz_2_5 = fd_z_2_5; dz_2_7 = fd_z_2_7; dz_3_4 = fd_z_3_4; dz_3_6 = fd_z_3_6; dz_4_6 = fd_z_4_6; dz_5_7 = fd_z_5_7;
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
    const double fd_x_0_2 = cm7;
    const double fd_x_0_5 = cm8;
    const double fd_x_0_7 = cm15;
    const double fd_x_1_3 = cm1;
    const double fd_x_1_4 = cm4;
    const double fd_x_1_6 = cm12;
    const double fd_x_2_5 = cm10;
    const double fd_x_2_7 = cm16;
    const double fd_x_3_4 = cm5;
    const double fd_x_3_6 = cm14;
    const double fd_x_4_6 = cm22;
    const double fd_x_5_7 = cm19;
    dx_0_2 = fd_x_0_2; dx_0_5 = fd_x_0_5; dx_0_7 = fd_x_0_7; dx_1_3 = fd_x_1_3; dx_1_4 = fd_x_1_4; dx_1_6 = fd_x_1_6; dx_2_5 = fd_x_2_5; dx_2_7 = fd_x_2_7; dx_3_4 = fd_x_3_4; dx_3_6 = fd_x_3_6; dx_4_6 = fd_x_4_6; dx_5_7 = fd_x_5_7;
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
    const double fd_y_0_2 = cm7;
    const double fd_y_0_5 = cm8;
    const double fd_y_0_7 = cm15;
    const double fd_y_1_3 = cm1;
    const double fd_y_1_4 = cm4;
    const double fd_y_1_6 = cm12;
    const double fd_y_2_5 = cm10;
    const double fd_y_2_7 = cm16;
    const double fd_y_3_4 = cm5;
    const double fd_y_3_6 = cm14;
    const double fd_y_4_6 = cm22;
    const double fd_y_5_7 = cm19;
    dy_0_2 = fd_y_0_2; dy_0_5 = fd_y_0_5; dy_0_7 = fd_y_0_7; dy_1_3 = fd_y_1_3; dy_1_4 = fd_y_1_4; dy_1_6 = fd_y_1_6; dy_2_5 = fd_y_2_5; dy_2_7 = fd_y_2_7; dy_3_4 = fd_y_3_4; dy_3_6 = fd_y_3_6; dy_4_6 = fd_y_4_6; dy_5_7 = fd_y_5_7;
  }
  if (CFL) {
    // squared distances (dx*dx + dy*dy) + dz*dz of time_integration.cpp:107-109,
    // pow(d, 2.0) == d*d; minimum taken on the order keys of the non-negative values
    long long kmin = 0x7FFFFFFFFFFFFFFFLL;
    { const double dx = (x[1] - x[0]), dy = (y[1] - y[0]), dz = (z[1] - z[0]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (0,1)
    { const double dx = (x[2] - x[1]), dy = (y[2] - y[1]), dz = (z[2] - z[1]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (1,2)
    { const double dx = (x[3] - x[2]), dy = (y[3] - y[2]), dz = (z[3] - z[2]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (2,3)
    { const double dx = dx_3_4, dy = dy_3_4, dz = dz_3_4;
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (3,4)
    { const double dx = (x[5] - x[4]), dy = (y[5] - y[4]), dz = (z[5] - z[4]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (4,5)
    { const double dx = (x[6] - x[5]), dy = (y[6] - y[5]), dz = (z[6] - z[5]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (5,6)
    { const double dx = (x[7] - x[6]), dy = (y[7] - y[6]), dz = (z[7] - z[6]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (6,7)
    { const double dx = dx_0_2, dy = dy_0_2, dz = dz_0_2;
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (0,2)
    { const double dx = dx_1_3, dy = dy_1_3, dz = dz_1_3;
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (1,3)
    { const double dx = (x[4] - x[2]), dy = (y[4] - y[2]), dz = (z[4] - z[2]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (2,4)
    { const double dx = (x[5] - x[3]), dy = (y[5] - y[3]), dz = (z[5] - z[3]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (3,5)
    { const double dx = dx_4_6, dy = dy_4_6, dz = dz_4_6;
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (4,6)
    { const double dx = dx_5_7, dy = dy_5_7, dz = dz_5_7;
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (5,7)
    { const double dx = (x[3] - x[0]), dy = (y[3] - y[0]), dz = (z[3] - z[0]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (0,3)
    { const double dx = dx_1_4, dy = dy_1_4, dz = dz_1_4;
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (1,4)
    { const double dx = dx_2_5, dy = dy_2_5, dz = dz_2_5;
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (2,5)
    { const double dx = dx_3_6, dy = dy_3_6, dz = dz_3_6;
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (3,6)
    { const double dx = (x[7] - x[4]), dy = (y[7] - y[4]), dz = (z[7] - z[4]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (4,7)
    { const double dx = (x[4] - x[0]), dy = (y[4] - y[0]), dz = (z[4] - z[0]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (0,4)
    { const double dx = (x[5] - x[1]), dy = (y[5] - y[1]), dz = (z[5] - z[1]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (1,5)
    { const double dx = (x[6] - x[2]), dy = (y[6] - y[2]), dz = (z[6] - z[2]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (2,6)
    { const double dx = (x[7] - x[3]), dy = (y[7] - y[3]), dz = (z[7] - z[3]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (3,7)
    { const double dx = dx_0_5, dy = dy_0_5, dz = dz_0_5;
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (0,5)
    { const double dx = dx_1_6, dy = dy_1_6, dz = dz_1_6;
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (1,6)
    { const double dx = dx_2_7, dy = dy_2_7, dz = dz_2_7;
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (2,7)
    { const double dx = (x[6] - x[0]), dy = (y[6] - y[0]), dz = (z[6] - z[0]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (0,6)
    { const double dx = (x[7] - x[1]), dy = (y[7] - y[1]), dz = (z[7] - z[1]);
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (1,7)
    { const double dx = dx_0_7, dy = dy_0_7, dz = dz_0_7;
      const double d2 = (dx * dx + dy * dy) + dz * dz;
      const long long k = okey(d2); kmin = k < kmin ? k : kmin; }  // pair (0,7)
    d2min = okey_decode(kmin);
  } else {
    d2min = 0.0;
    (void)(dz_0_2 + dz_0_5 + dz_0_7 + dz_1_3 + dz_1_4 + dz_1_6 + dz_2_5 + dz_2_7 + dz_3_4 + dz_3_6 + dz_4_6 + dz_5_7 + dx_0_2 + dx_0_5 + dx_0_7 + dx_1_3 + dx_1_4 + dx_1_6 + dx_2_5 + dx_2_7 + dx_3_4 + dx_3_6 + dx_4_6 + dx_5_7 + dy_0_2 + dy_0_5 + dy_0_7 + dy_1_3 + dy_1_4 + dy_1_6 + dy_2_5 + dy_2_7 + dy_3_4 + dy_3_6 + dy_4_6 + dy_5_7);
  }
}
