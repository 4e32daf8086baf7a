/* Generated by oracle/codegen_ref.py -- do not edit.
 * Straight-line codelets restating recmo/goldilocks ntt/src/ntt/small.rs
 * (as produced by ntt/src/bin/codegen.rs), in canonical representation.
 * Test infrastructure only (CPU oracle). */
#include "gl_oracle_internal.h"

static void o_ntt_2(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1];
    { uint64_t t1 = a0; a0 = o_add(t1, a1); a1 = o_sub(t1, a1); }
    v[0] = a0;
    v[1] = a1;
}

static void o_ntt_3(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2];
    { uint64_t t1 = a0, t2 = a1, t3 = a2;
      a0 = o_add(o_add(t1, t2), t3);
      a1 = o_sub(o_add(t1, o_shift(t2, 64)), o_shift(t3, 32));
      a2 = o_add(o_sub(t1, o_shift(t2, 32)), o_shift(t3, 64)); }
    v[0] = a0;
    v[1] = a1;
    v[2] = a2;
}

static void o_ntt_4(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3];
    { uint64_t t1 = a0; a0 = o_add(t1, a2); a2 = o_sub(t1, a2); }
    { uint64_t t2 = a1; a1 = o_add(t2, a3); a3 = o_sub(t2, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t3 = a0; a0 = o_add(t3, a1); a1 = o_sub(t3, a1); }
    { uint64_t t4 = a2; a2 = o_add(t4, a3); a3 = o_sub(t4, a3); }
    v[0] = a0;
    v[1] = a2;
    v[2] = a1;
    v[3] = a3;
}

static void o_ntt_5(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4];
    { uint64_t t1 = a1; a1 = o_add(t1, a4); a4 = o_sub(t1, a4); }
    { uint64_t t2 = a3; a3 = o_add(t2, a2); a2 = o_sub(t2, a2); }
    a2 = o_shift(a2, 48);
    { uint64_t t3 = a1; a1 = o_add(t3, a3); a3 = o_sub(t3, a3); }
    { uint64_t t4 = a4; a4 = o_add(t4, a2); a2 = o_sub(t4, a2); }
    uint64_t t5 = a0;
    a0 = o_add(a0, a1);
    a1 = o_mul(a1, 4611686017353646080ULL);
    a4 = o_mul(a4, 16181989089180173841ULL);
    a3 = o_mul(a3, 5818851782451133869ULL);
    a2 = o_mul(a2, 11322249509082494407ULL);
    a1 = o_add(a1, t5);
    { uint64_t t6 = a1; a1 = o_add(t6, a3); a3 = o_sub(t6, a3); }
    { uint64_t t7 = a2; a2 = o_add(t7, a4); a4 = o_sub(t7, a4); }
    a4 = o_shift(a4, 48);
    { uint64_t t8 = a1; a1 = o_add(t8, a2); a2 = o_sub(t8, a2); }
    { uint64_t t9 = a3; a3 = o_add(t9, a4); a4 = o_sub(t9, a4); }
    v[0] = a0;
    v[1] = a1;
    v[2] = a3;
    v[3] = a4;
    v[4] = a2;
}

static void o_ntt_6(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5];
    { uint64_t t1 = a0, t2 = a2, t3 = a4;
      a0 = o_add(o_add(t1, t2), t3);
      a2 = o_sub(o_add(t1, o_shift(t2, 64)), o_shift(t3, 32));
      a4 = o_add(o_sub(t1, o_shift(t2, 32)), o_shift(t3, 64)); }
    { uint64_t t4 = a3, t5 = a5, t6 = a1;
      a3 = o_add(o_add(t4, t5), t6);
      a5 = o_sub(o_add(t4, o_shift(t5, 64)), o_shift(t6, 32));
      a1 = o_add(o_sub(t4, o_shift(t5, 32)), o_shift(t6, 64)); }
    { uint64_t t7 = a0; a0 = o_add(t7, a3); a3 = o_sub(t7, a3); }
    { uint64_t t8 = a2; a2 = o_add(t8, a5); a5 = o_sub(t8, a5); }
    { uint64_t t9 = a4; a4 = o_add(t9, a1); a1 = o_sub(t9, a1); }
    v[0] = a0;
    v[1] = a5;
    v[2] = a4;
    v[3] = a3;
    v[4] = a2;
    v[5] = a1;
}

static void o_ntt_8(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7];
    { uint64_t t1 = a0; a0 = o_add(t1, a4); a4 = o_sub(t1, a4); }
    { uint64_t t2 = a1; a1 = o_add(t2, a5); a5 = o_sub(t2, a5); }
    { uint64_t t3 = a2; a2 = o_add(t3, a6); a6 = o_sub(t3, a6); }
    { uint64_t t4 = a3; a3 = o_add(t4, a7); a7 = o_sub(t4, a7); }
    a5 = o_shift(a5, 24);
    a6 = o_shift(a6, 48);
    a7 = o_shift(a7, 72);
    { uint64_t t5 = a0; a0 = o_add(t5, a2); a2 = o_sub(t5, a2); }
    { uint64_t t6 = a1; a1 = o_add(t6, a3); a3 = o_sub(t6, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t7 = a0; a0 = o_add(t7, a1); a1 = o_sub(t7, a1); }
    { uint64_t t8 = a2; a2 = o_add(t8, a3); a3 = o_sub(t8, a3); }
    { uint64_t t9 = a4; a4 = o_add(t9, a6); a6 = o_sub(t9, a6); }
    { uint64_t t10 = a5; a5 = o_add(t10, a7); a7 = o_sub(t10, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t11 = a4; a4 = o_add(t11, a5); a5 = o_sub(t11, a5); }
    { uint64_t t12 = a6; a6 = o_add(t12, a7); a7 = o_sub(t12, a7); }
    v[0] = a0;
    v[1] = a4;
    v[2] = a2;
    v[3] = a6;
    v[4] = a1;
    v[5] = a5;
    v[6] = a3;
    v[7] = a7;
}

static void o_ntt_10(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9];
    { uint64_t t1 = a2; a2 = o_add(t1, a8); a8 = o_sub(t1, a8); }
    { uint64_t t2 = a6; a6 = o_add(t2, a4); a4 = o_sub(t2, a4); }
    a4 = o_shift(a4, 48);
    { uint64_t t3 = a2; a2 = o_add(t3, a6); a6 = o_sub(t3, a6); }
    { uint64_t t4 = a8; a8 = o_add(t4, a4); a4 = o_sub(t4, a4); }
    uint64_t t5 = a0;
    a0 = o_add(a0, a2);
    a2 = o_mul(a2, 4611686017353646080ULL);
    a8 = o_mul(a8, 16181989089180173841ULL);
    a6 = o_mul(a6, 5818851782451133869ULL);
    a4 = o_mul(a4, 11322249509082494407ULL);
    a2 = o_add(a2, t5);
    { uint64_t t6 = a2; a2 = o_add(t6, a6); a6 = o_sub(t6, a6); }
    { uint64_t t7 = a4; a4 = o_add(t7, a8); a8 = o_sub(t7, a8); }
    a8 = o_shift(a8, 48);
    { uint64_t t8 = a2; a2 = o_add(t8, a4); a4 = o_sub(t8, a4); }
    { uint64_t t9 = a6; a6 = o_add(t9, a8); a8 = o_sub(t9, a8); }
    { uint64_t t10 = a7; a7 = o_add(t10, a3); a3 = o_sub(t10, a3); }
    { uint64_t t11 = a1; a1 = o_add(t11, a9); a9 = o_sub(t11, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t12 = a7; a7 = o_add(t12, a1); a1 = o_sub(t12, a1); }
    { uint64_t t13 = a3; a3 = o_add(t13, a9); a9 = o_sub(t13, a9); }
    uint64_t t14 = a5;
    a5 = o_add(a5, a7);
    a7 = o_mul(a7, 4611686017353646080ULL);
    a3 = o_mul(a3, 16181989089180173841ULL);
    a1 = o_mul(a1, 5818851782451133869ULL);
    a9 = o_mul(a9, 11322249509082494407ULL);
    a7 = o_add(a7, t14);
    { uint64_t t15 = a7; a7 = o_add(t15, a1); a1 = o_sub(t15, a1); }
    { uint64_t t16 = a9; a9 = o_add(t16, a3); a3 = o_sub(t16, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t17 = a7; a7 = o_add(t17, a9); a9 = o_sub(t17, a9); }
    { uint64_t t18 = a1; a1 = o_add(t18, a3); a3 = o_sub(t18, a3); }
    { uint64_t t19 = a0; a0 = o_add(t19, a5); a5 = o_sub(t19, a5); }
    { uint64_t t20 = a2; a2 = o_add(t20, a7); a7 = o_sub(t20, a7); }
    { uint64_t t21 = a6; a6 = o_add(t21, a1); a1 = o_sub(t21, a1); }
    { uint64_t t22 = a8; a8 = o_add(t22, a3); a3 = o_sub(t22, a3); }
    { uint64_t t23 = a4; a4 = o_add(t23, a9); a9 = o_sub(t23, a9); }
    v[0] = a0;
    v[1] = a7;
    v[2] = a6;
    v[3] = a3;
    v[4] = a4;
    v[5] = a5;
    v[6] = a2;
    v[7] = a1;
    v[8] = a8;
    v[9] = a9;
}

static void o_ntt_12(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11];
    { uint64_t t1 = a0; a0 = o_add(t1, a6); a6 = o_sub(t1, a6); }
    { uint64_t t2 = a3; a3 = o_add(t2, a9); a9 = o_sub(t2, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t3 = a0; a0 = o_add(t3, a3); a3 = o_sub(t3, a3); }
    { uint64_t t4 = a6; a6 = o_add(t4, a9); a9 = o_sub(t4, a9); }
    { uint64_t t5 = a4; a4 = o_add(t5, a10); a10 = o_sub(t5, a10); }
    { uint64_t t6 = a7; a7 = o_add(t6, a1); a1 = o_sub(t6, a1); }
    a1 = o_shift(a1, 48);
    { uint64_t t7 = a4; a4 = o_add(t7, a7); a7 = o_sub(t7, a7); }
    { uint64_t t8 = a10; a10 = o_add(t8, a1); a1 = o_sub(t8, a1); }
    { uint64_t t9 = a8; a8 = o_add(t9, a2); a2 = o_sub(t9, a2); }
    { uint64_t t10 = a11; a11 = o_add(t10, a5); a5 = o_sub(t10, a5); }
    a5 = o_shift(a5, 48);
    { uint64_t t11 = a8; a8 = o_add(t11, a11); a11 = o_sub(t11, a11); }
    { uint64_t t12 = a2; a2 = o_add(t12, a5); a5 = o_sub(t12, a5); }
    { uint64_t t13 = a0, t14 = a4, t15 = a8;
      a0 = o_add(o_add(t13, t14), t15);
      a4 = o_sub(o_add(t13, o_shift(t14, 64)), o_shift(t15, 32));
      a8 = o_add(o_sub(t13, o_shift(t14, 32)), o_shift(t15, 64)); }
    { uint64_t t16 = a6, t17 = a10, t18 = a2;
      a6 = o_add(o_add(t16, t17), t18);
      a10 = o_sub(o_add(t16, o_shift(t17, 64)), o_shift(t18, 32));
      a2 = o_add(o_sub(t16, o_shift(t17, 32)), o_shift(t18, 64)); }
    { uint64_t t19 = a3, t20 = a7, t21 = a11;
      a3 = o_add(o_add(t19, t20), t21);
      a7 = o_sub(o_add(t19, o_shift(t20, 64)), o_shift(t21, 32));
      a11 = o_add(o_sub(t19, o_shift(t20, 32)), o_shift(t21, 64)); }
    { uint64_t t22 = a9, t23 = a1, t24 = a5;
      a9 = o_add(o_add(t22, t23), t24);
      a1 = o_sub(o_add(t22, o_shift(t23, 64)), o_shift(t24, 32));
      a5 = o_add(o_sub(t22, o_shift(t23, 32)), o_shift(t24, 64)); }
    v[0] = a0;
    v[1] = a10;
    v[2] = a11;
    v[3] = a9;
    v[4] = a4;
    v[5] = a2;
    v[6] = a3;
    v[7] = a1;
    v[8] = a8;
    v[9] = a6;
    v[10] = a7;
    v[11] = a5;
}

static void o_ntt_15(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14];
    { uint64_t t1 = a3; a3 = o_add(t1, a12); a12 = o_sub(t1, a12); }
    { uint64_t t2 = a9; a9 = o_add(t2, a6); a6 = o_sub(t2, a6); }
    a6 = o_shift(a6, 48);
    { uint64_t t3 = a3; a3 = o_add(t3, a9); a9 = o_sub(t3, a9); }
    { uint64_t t4 = a12; a12 = o_add(t4, a6); a6 = o_sub(t4, a6); }
    uint64_t t5 = a0;
    a0 = o_add(a0, a3);
    a3 = o_mul(a3, 4611686017353646080ULL);
    a12 = o_mul(a12, 16181989089180173841ULL);
    a9 = o_mul(a9, 5818851782451133869ULL);
    a6 = o_mul(a6, 11322249509082494407ULL);
    a3 = o_add(a3, t5);
    { uint64_t t6 = a3; a3 = o_add(t6, a9); a9 = o_sub(t6, a9); }
    { uint64_t t7 = a6; a6 = o_add(t7, a12); a12 = o_sub(t7, a12); }
    a12 = o_shift(a12, 48);
    { uint64_t t8 = a3; a3 = o_add(t8, a6); a6 = o_sub(t8, a6); }
    { uint64_t t9 = a9; a9 = o_add(t9, a12); a12 = o_sub(t9, a12); }
    { uint64_t t10 = a8; a8 = o_add(t10, a2); a2 = o_sub(t10, a2); }
    { uint64_t t11 = a14; a14 = o_add(t11, a11); a11 = o_sub(t11, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t12 = a8; a8 = o_add(t12, a14); a14 = o_sub(t12, a14); }
    { uint64_t t13 = a2; a2 = o_add(t13, a11); a11 = o_sub(t13, a11); }
    uint64_t t14 = a5;
    a5 = o_add(a5, a8);
    a8 = o_mul(a8, 4611686017353646080ULL);
    a2 = o_mul(a2, 16181989089180173841ULL);
    a14 = o_mul(a14, 5818851782451133869ULL);
    a11 = o_mul(a11, 11322249509082494407ULL);
    a8 = o_add(a8, t14);
    { uint64_t t15 = a8; a8 = o_add(t15, a14); a14 = o_sub(t15, a14); }
    { uint64_t t16 = a11; a11 = o_add(t16, a2); a2 = o_sub(t16, a2); }
    a2 = o_shift(a2, 48);
    { uint64_t t17 = a8; a8 = o_add(t17, a11); a11 = o_sub(t17, a11); }
    { uint64_t t18 = a14; a14 = o_add(t18, a2); a2 = o_sub(t18, a2); }
    { uint64_t t19 = a13; a13 = o_add(t19, a7); a7 = o_sub(t19, a7); }
    { uint64_t t20 = a4; a4 = o_add(t20, a1); a1 = o_sub(t20, a1); }
    a1 = o_shift(a1, 48);
    { uint64_t t21 = a13; a13 = o_add(t21, a4); a4 = o_sub(t21, a4); }
    { uint64_t t22 = a7; a7 = o_add(t22, a1); a1 = o_sub(t22, a1); }
    uint64_t t23 = a10;
    a10 = o_add(a10, a13);
    a13 = o_mul(a13, 4611686017353646080ULL);
    a7 = o_mul(a7, 16181989089180173841ULL);
    a4 = o_mul(a4, 5818851782451133869ULL);
    a1 = o_mul(a1, 11322249509082494407ULL);
    a13 = o_add(a13, t23);
    { uint64_t t24 = a13; a13 = o_add(t24, a4); a4 = o_sub(t24, a4); }
    { uint64_t t25 = a1; a1 = o_add(t25, a7); a7 = o_sub(t25, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t26 = a13; a13 = o_add(t26, a1); a1 = o_sub(t26, a1); }
    { uint64_t t27 = a4; a4 = o_add(t27, a7); a7 = o_sub(t27, a7); }
    { uint64_t t28 = a0, t29 = a5, t30 = a10;
      a0 = o_add(o_add(t28, t29), t30);
      a5 = o_sub(o_add(t28, o_shift(t29, 64)), o_shift(t30, 32));
      a10 = o_add(o_sub(t28, o_shift(t29, 32)), o_shift(t30, 64)); }
    { uint64_t t31 = a3, t32 = a8, t33 = a13;
      a3 = o_add(o_add(t31, t32), t33);
      a8 = o_sub(o_add(t31, o_shift(t32, 64)), o_shift(t33, 32));
      a13 = o_add(o_sub(t31, o_shift(t32, 32)), o_shift(t33, 64)); }
    { uint64_t t34 = a9, t35 = a14, t36 = a4;
      a9 = o_add(o_add(t34, t35), t36);
      a14 = o_sub(o_add(t34, o_shift(t35, 64)), o_shift(t36, 32));
      a4 = o_add(o_sub(t34, o_shift(t35, 32)), o_shift(t36, 64)); }
    { uint64_t t37 = a12, t38 = a2, t39 = a7;
      a12 = o_add(o_add(t37, t38), t39);
      a2 = o_sub(o_add(t37, o_shift(t38, 64)), o_shift(t39, 32));
      a7 = o_add(o_sub(t37, o_shift(t38, 32)), o_shift(t39, 64)); }
    { uint64_t t40 = a6, t41 = a11, t42 = a1;
      a6 = o_add(o_add(t40, t41), t42);
      a11 = o_sub(o_add(t40, o_shift(t41, 64)), o_shift(t42, 32));
      a1 = o_add(o_sub(t40, o_shift(t41, 32)), o_shift(t42, 64)); }
    v[0] = a0;
    v[1] = a8;
    v[2] = a4;
    v[3] = a12;
    v[4] = a11;
    v[5] = a10;
    v[6] = a3;
    v[7] = a14;
    v[8] = a7;
    v[9] = a6;
    v[10] = a5;
    v[11] = a13;
    v[12] = a9;
    v[13] = a2;
    v[14] = a1;
}

static void o_ntt_16(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15];
    { uint64_t t1 = a0; a0 = o_add(t1, a8); a8 = o_sub(t1, a8); }
    { uint64_t t2 = a4; a4 = o_add(t2, a12); a12 = o_sub(t2, a12); }
    a12 = o_shift(a12, 48);
    { uint64_t t3 = a0; a0 = o_add(t3, a4); a4 = o_sub(t3, a4); }
    { uint64_t t4 = a8; a8 = o_add(t4, a12); a12 = o_sub(t4, a12); }
    { uint64_t t5 = a1; a1 = o_add(t5, a9); a9 = o_sub(t5, a9); }
    { uint64_t t6 = a5; a5 = o_add(t6, a13); a13 = o_sub(t6, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t7 = a1; a1 = o_add(t7, a5); a5 = o_sub(t7, a5); }
    { uint64_t t8 = a9; a9 = o_add(t8, a13); a13 = o_sub(t8, a13); }
    { uint64_t t9 = a2; a2 = o_add(t9, a10); a10 = o_sub(t9, a10); }
    { uint64_t t10 = a6; a6 = o_add(t10, a14); a14 = o_sub(t10, a14); }
    a14 = o_shift(a14, 48);
    { uint64_t t11 = a2; a2 = o_add(t11, a6); a6 = o_sub(t11, a6); }
    { uint64_t t12 = a10; a10 = o_add(t12, a14); a14 = o_sub(t12, a14); }
    { uint64_t t13 = a3; a3 = o_add(t13, a11); a11 = o_sub(t13, a11); }
    { uint64_t t14 = a7; a7 = o_add(t14, a15); a15 = o_sub(t14, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t15 = a3; a3 = o_add(t15, a7); a7 = o_sub(t15, a7); }
    { uint64_t t16 = a11; a11 = o_add(t16, a15); a15 = o_sub(t16, a15); }
    a9 = o_shift(a9, 12);
    a5 = o_shift(a5, 24);
    a13 = o_shift(a13, 36);
    a10 = o_shift(a10, 24);
    a6 = o_shift(a6, 48);
    a14 = o_shift(a14, 72);
    a11 = o_shift(a11, 36);
    a7 = o_shift(a7, 72);
    a15 = o_neg(o_shift(a15, 12));
    { uint64_t t17 = a0; a0 = o_add(t17, a2); a2 = o_sub(t17, a2); }
    { uint64_t t18 = a1; a1 = o_add(t18, a3); a3 = o_sub(t18, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t19 = a0; a0 = o_add(t19, a1); a1 = o_sub(t19, a1); }
    { uint64_t t20 = a2; a2 = o_add(t20, a3); a3 = o_sub(t20, a3); }
    { uint64_t t21 = a8; a8 = o_add(t21, a10); a10 = o_sub(t21, a10); }
    { uint64_t t22 = a9; a9 = o_add(t22, a11); a11 = o_sub(t22, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t23 = a8; a8 = o_add(t23, a9); a9 = o_sub(t23, a9); }
    { uint64_t t24 = a10; a10 = o_add(t24, a11); a11 = o_sub(t24, a11); }
    { uint64_t t25 = a4; a4 = o_add(t25, a6); a6 = o_sub(t25, a6); }
    { uint64_t t26 = a5; a5 = o_add(t26, a7); a7 = o_sub(t26, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t27 = a4; a4 = o_add(t27, a5); a5 = o_sub(t27, a5); }
    { uint64_t t28 = a6; a6 = o_add(t28, a7); a7 = o_sub(t28, a7); }
    { uint64_t t29 = a12; a12 = o_add(t29, a14); a14 = o_sub(t29, a14); }
    { uint64_t t30 = a13; a13 = o_add(t30, a15); a15 = o_sub(t30, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t31 = a12; a12 = o_add(t31, a13); a13 = o_sub(t31, a13); }
    { uint64_t t32 = a14; a14 = o_add(t32, a15); a15 = o_sub(t32, a15); }
    v[0] = a0;
    v[1] = a8;
    v[2] = a4;
    v[3] = a12;
    v[4] = a2;
    v[5] = a10;
    v[6] = a6;
    v[7] = a14;
    v[8] = a1;
    v[9] = a9;
    v[10] = a5;
    v[11] = a13;
    v[12] = a3;
    v[13] = a11;
    v[14] = a7;
    v[15] = a15;
}

static void o_ntt_17(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16];
    { uint64_t t1 = a1; a1 = o_add(t1, a16); a16 = o_sub(t1, a16); }
    { uint64_t t2 = a4; a4 = o_add(t2, a13); a13 = o_sub(t2, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t3 = a1; a1 = o_add(t3, a4); a4 = o_sub(t3, a4); }
    { uint64_t t4 = a16; a16 = o_add(t4, a13); a13 = o_sub(t4, a13); }
    { uint64_t t5 = a6; a6 = o_add(t5, a11); a11 = o_sub(t5, a11); }
    { uint64_t t6 = a7; a7 = o_add(t6, a10); a10 = o_sub(t6, a10); }
    a10 = o_shift(a10, 48);
    { uint64_t t7 = a6; a6 = o_add(t7, a7); a7 = o_sub(t7, a7); }
    { uint64_t t8 = a11; a11 = o_add(t8, a10); a10 = o_sub(t8, a10); }
    { uint64_t t9 = a2; a2 = o_add(t9, a15); a15 = o_sub(t9, a15); }
    { uint64_t t10 = a8; a8 = o_add(t10, a9); a9 = o_sub(t10, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t11 = a2; a2 = o_add(t11, a8); a8 = o_sub(t11, a8); }
    { uint64_t t12 = a15; a15 = o_add(t12, a9); a9 = o_sub(t12, a9); }
    { uint64_t t13 = a12; a12 = o_add(t13, a5); a5 = o_sub(t13, a5); }
    { uint64_t t14 = a14; a14 = o_add(t14, a3); a3 = o_sub(t14, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t15 = a12; a12 = o_add(t15, a14); a14 = o_sub(t15, a14); }
    { uint64_t t16 = a5; a5 = o_add(t16, a3); a3 = o_sub(t16, a3); }
    a11 = o_shift(a11, 12);
    a7 = o_shift(a7, 24);
    a10 = o_shift(a10, 36);
    a15 = o_shift(a15, 24);
    a8 = o_shift(a8, 48);
    a9 = o_shift(a9, 72);
    a5 = o_shift(a5, 36);
    a14 = o_shift(a14, 72);
    a3 = o_neg(o_shift(a3, 12));
    { uint64_t t17 = a1; a1 = o_add(t17, a2); a2 = o_sub(t17, a2); }
    { uint64_t t18 = a6; a6 = o_add(t18, a12); a12 = o_sub(t18, a12); }
    a12 = o_shift(a12, 48);
    { uint64_t t19 = a1; a1 = o_add(t19, a6); a6 = o_sub(t19, a6); }
    { uint64_t t20 = a2; a2 = o_add(t20, a12); a12 = o_sub(t20, a12); }
    { uint64_t t21 = a16; a16 = o_add(t21, a15); a15 = o_sub(t21, a15); }
    { uint64_t t22 = a11; a11 = o_add(t22, a5); a5 = o_sub(t22, a5); }
    a5 = o_shift(a5, 48);
    { uint64_t t23 = a16; a16 = o_add(t23, a11); a11 = o_sub(t23, a11); }
    { uint64_t t24 = a15; a15 = o_add(t24, a5); a5 = o_sub(t24, a5); }
    { uint64_t t25 = a4; a4 = o_add(t25, a8); a8 = o_sub(t25, a8); }
    { uint64_t t26 = a7; a7 = o_add(t26, a14); a14 = o_sub(t26, a14); }
    a14 = o_shift(a14, 48);
    { uint64_t t27 = a4; a4 = o_add(t27, a7); a7 = o_sub(t27, a7); }
    { uint64_t t28 = a8; a8 = o_add(t28, a14); a14 = o_sub(t28, a14); }
    { uint64_t t29 = a13; a13 = o_add(t29, a9); a9 = o_sub(t29, a9); }
    { uint64_t t30 = a10; a10 = o_add(t30, a3); a3 = o_sub(t30, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t31 = a13; a13 = o_add(t31, a10); a10 = o_sub(t31, a10); }
    { uint64_t t32 = a9; a9 = o_add(t32, a3); a3 = o_sub(t32, a3); }
    uint64_t t33 = a0;
    a0 = o_add(a0, a1);
    a1 = o_mul(a1, 1152921504338411520ULL);
    a16 = o_mul(a16, 6259776822214049175ULL);
    a4 = o_mul(a4, 9380094172986290191ULL);
    a13 = o_mul(a13, 891943630314919127ULL);
    a2 = o_mul(a2, 17228171707553225791ULL);
    a15 = o_mul(a15, 12855743360534130886ULL);
    a8 = o_mul(a8, 6167687396920564837ULL);
    a9 = o_mul(a9, 17201834061724655524ULL);
    a6 = o_mul(a6, 15308299771656910737ULL);
    a11 = o_mul(a11, 18186005861103657533ULL);
    a7 = o_mul(a7, 53595491891823545ULL);
    a10 = o_mul(a10, 1906638201581172103ULL);
    a12 = o_mul(a12, 18303651001328874822ULL);
    a5 = o_mul(a5, 3077466521755967626ULL);
    a14 = o_mul(a14, 12423593102987598328ULL);
    a3 = o_mul(a3, 18361513053649472048ULL);
    a1 = o_add(a1, t33);
    { uint64_t t34 = a1; a1 = o_add(t34, a6); a6 = o_sub(t34, a6); }
    { uint64_t t35 = a12; a12 = o_add(t35, a2); a2 = o_sub(t35, a2); }
    a2 = o_shift(a2, 48);
    { uint64_t t36 = a1; a1 = o_add(t36, a12); a12 = o_sub(t36, a12); }
    { uint64_t t37 = a6; a6 = o_add(t37, a2); a2 = o_sub(t37, a2); }
    { uint64_t t38 = a3; a3 = o_add(t38, a9); a9 = o_sub(t38, a9); }
    { uint64_t t39 = a10; a10 = o_add(t39, a13); a13 = o_sub(t39, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t40 = a3; a3 = o_add(t40, a10); a10 = o_sub(t40, a10); }
    { uint64_t t41 = a9; a9 = o_add(t41, a13); a13 = o_sub(t41, a13); }
    { uint64_t t42 = a14; a14 = o_add(t42, a8); a8 = o_sub(t42, a8); }
    { uint64_t t43 = a7; a7 = o_add(t43, a4); a4 = o_sub(t43, a4); }
    a4 = o_shift(a4, 48);
    { uint64_t t44 = a14; a14 = o_add(t44, a7); a7 = o_sub(t44, a7); }
    { uint64_t t45 = a8; a8 = o_add(t45, a4); a4 = o_sub(t45, a4); }
    { uint64_t t46 = a5; a5 = o_add(t46, a15); a15 = o_sub(t46, a15); }
    { uint64_t t47 = a11; a11 = o_add(t47, a16); a16 = o_sub(t47, a16); }
    a16 = o_shift(a16, 48);
    { uint64_t t48 = a5; a5 = o_add(t48, a11); a11 = o_sub(t48, a11); }
    { uint64_t t49 = a15; a15 = o_add(t49, a16); a16 = o_sub(t49, a16); }
    a9 = o_shift(a9, 12);
    a10 = o_shift(a10, 24);
    a13 = o_shift(a13, 36);
    a8 = o_shift(a8, 24);
    a7 = o_shift(a7, 48);
    a4 = o_shift(a4, 72);
    a15 = o_shift(a15, 36);
    a11 = o_shift(a11, 72);
    a16 = o_neg(o_shift(a16, 12));
    { uint64_t t50 = a1; a1 = o_add(t50, a14); a14 = o_sub(t50, a14); }
    { uint64_t t51 = a3; a3 = o_add(t51, a5); a5 = o_sub(t51, a5); }
    a5 = o_shift(a5, 48);
    { uint64_t t52 = a1; a1 = o_add(t52, a3); a3 = o_sub(t52, a3); }
    { uint64_t t53 = a14; a14 = o_add(t53, a5); a5 = o_sub(t53, a5); }
    { uint64_t t54 = a6; a6 = o_add(t54, a8); a8 = o_sub(t54, a8); }
    { uint64_t t55 = a9; a9 = o_add(t55, a15); a15 = o_sub(t55, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t56 = a6; a6 = o_add(t56, a9); a9 = o_sub(t56, a9); }
    { uint64_t t57 = a8; a8 = o_add(t57, a15); a15 = o_sub(t57, a15); }
    { uint64_t t58 = a12; a12 = o_add(t58, a7); a7 = o_sub(t58, a7); }
    { uint64_t t59 = a10; a10 = o_add(t59, a11); a11 = o_sub(t59, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t60 = a12; a12 = o_add(t60, a10); a10 = o_sub(t60, a10); }
    { uint64_t t61 = a7; a7 = o_add(t61, a11); a11 = o_sub(t61, a11); }
    { uint64_t t62 = a2; a2 = o_add(t62, a4); a4 = o_sub(t62, a4); }
    { uint64_t t63 = a13; a13 = o_add(t63, a16); a16 = o_sub(t63, a16); }
    a16 = o_shift(a16, 48);
    { uint64_t t64 = a2; a2 = o_add(t64, a13); a13 = o_sub(t64, a13); }
    { uint64_t t65 = a4; a4 = o_add(t65, a16); a16 = o_sub(t65, a16); }
    v[0] = a0;
    v[1] = a1;
    v[2] = a11;
    v[3] = a6;
    v[4] = a5;
    v[5] = a8;
    v[6] = a16;
    v[7] = a13;
    v[8] = a10;
    v[9] = a12;
    v[10] = a2;
    v[11] = a4;
    v[12] = a15;
    v[13] = a14;
    v[14] = a9;
    v[15] = a7;
    v[16] = a3;
}

static void o_ntt_20(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19];
    { uint64_t t1 = a4; a4 = o_add(t1, a16); a16 = o_sub(t1, a16); }
    { uint64_t t2 = a12; a12 = o_add(t2, a8); a8 = o_sub(t2, a8); }
    a8 = o_shift(a8, 48);
    { uint64_t t3 = a4; a4 = o_add(t3, a12); a12 = o_sub(t3, a12); }
    { uint64_t t4 = a16; a16 = o_add(t4, a8); a8 = o_sub(t4, a8); }
    uint64_t t5 = a0;
    a0 = o_add(a0, a4);
    a4 = o_mul(a4, 4611686017353646080ULL);
    a16 = o_mul(a16, 16181989089180173841ULL);
    a12 = o_mul(a12, 5818851782451133869ULL);
    a8 = o_mul(a8, 11322249509082494407ULL);
    a4 = o_add(a4, t5);
    { uint64_t t6 = a4; a4 = o_add(t6, a12); a12 = o_sub(t6, a12); }
    { uint64_t t7 = a8; a8 = o_add(t7, a16); a16 = o_sub(t7, a16); }
    a16 = o_shift(a16, 48);
    { uint64_t t8 = a4; a4 = o_add(t8, a8); a8 = o_sub(t8, a8); }
    { uint64_t t9 = a12; a12 = o_add(t9, a16); a16 = o_sub(t9, a16); }
    { uint64_t t10 = a9; a9 = o_add(t10, a1); a1 = o_sub(t10, a1); }
    { uint64_t t11 = a17; a17 = o_add(t11, a13); a13 = o_sub(t11, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t12 = a9; a9 = o_add(t12, a17); a17 = o_sub(t12, a17); }
    { uint64_t t13 = a1; a1 = o_add(t13, a13); a13 = o_sub(t13, a13); }
    uint64_t t14 = a5;
    a5 = o_add(a5, a9);
    a9 = o_mul(a9, 4611686017353646080ULL);
    a1 = o_mul(a1, 16181989089180173841ULL);
    a17 = o_mul(a17, 5818851782451133869ULL);
    a13 = o_mul(a13, 11322249509082494407ULL);
    a9 = o_add(a9, t14);
    { uint64_t t15 = a9; a9 = o_add(t15, a17); a17 = o_sub(t15, a17); }
    { uint64_t t16 = a13; a13 = o_add(t16, a1); a1 = o_sub(t16, a1); }
    a1 = o_shift(a1, 48);
    { uint64_t t17 = a9; a9 = o_add(t17, a13); a13 = o_sub(t17, a13); }
    { uint64_t t18 = a17; a17 = o_add(t18, a1); a1 = o_sub(t18, a1); }
    { uint64_t t19 = a14; a14 = o_add(t19, a6); a6 = o_sub(t19, a6); }
    { uint64_t t20 = a2; a2 = o_add(t20, a18); a18 = o_sub(t20, a18); }
    a18 = o_shift(a18, 48);
    { uint64_t t21 = a14; a14 = o_add(t21, a2); a2 = o_sub(t21, a2); }
    { uint64_t t22 = a6; a6 = o_add(t22, a18); a18 = o_sub(t22, a18); }
    uint64_t t23 = a10;
    a10 = o_add(a10, a14);
    a14 = o_mul(a14, 4611686017353646080ULL);
    a6 = o_mul(a6, 16181989089180173841ULL);
    a2 = o_mul(a2, 5818851782451133869ULL);
    a18 = o_mul(a18, 11322249509082494407ULL);
    a14 = o_add(a14, t23);
    { uint64_t t24 = a14; a14 = o_add(t24, a2); a2 = o_sub(t24, a2); }
    { uint64_t t25 = a18; a18 = o_add(t25, a6); a6 = o_sub(t25, a6); }
    a6 = o_shift(a6, 48);
    { uint64_t t26 = a14; a14 = o_add(t26, a18); a18 = o_sub(t26, a18); }
    { uint64_t t27 = a2; a2 = o_add(t27, a6); a6 = o_sub(t27, a6); }
    { uint64_t t28 = a19; a19 = o_add(t28, a11); a11 = o_sub(t28, a11); }
    { uint64_t t29 = a7; a7 = o_add(t29, a3); a3 = o_sub(t29, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t30 = a19; a19 = o_add(t30, a7); a7 = o_sub(t30, a7); }
    { uint64_t t31 = a11; a11 = o_add(t31, a3); a3 = o_sub(t31, a3); }
    uint64_t t32 = a15;
    a15 = o_add(a15, a19);
    a19 = o_mul(a19, 4611686017353646080ULL);
    a11 = o_mul(a11, 16181989089180173841ULL);
    a7 = o_mul(a7, 5818851782451133869ULL);
    a3 = o_mul(a3, 11322249509082494407ULL);
    a19 = o_add(a19, t32);
    { uint64_t t33 = a19; a19 = o_add(t33, a7); a7 = o_sub(t33, a7); }
    { uint64_t t34 = a3; a3 = o_add(t34, a11); a11 = o_sub(t34, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t35 = a19; a19 = o_add(t35, a3); a3 = o_sub(t35, a3); }
    { uint64_t t36 = a7; a7 = o_add(t36, a11); a11 = o_sub(t36, a11); }
    { uint64_t t37 = a0; a0 = o_add(t37, a10); a10 = o_sub(t37, a10); }
    { uint64_t t38 = a5; a5 = o_add(t38, a15); a15 = o_sub(t38, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t39 = a0; a0 = o_add(t39, a5); a5 = o_sub(t39, a5); }
    { uint64_t t40 = a10; a10 = o_add(t40, a15); a15 = o_sub(t40, a15); }
    { uint64_t t41 = a4; a4 = o_add(t41, a14); a14 = o_sub(t41, a14); }
    { uint64_t t42 = a9; a9 = o_add(t42, a19); a19 = o_sub(t42, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t43 = a4; a4 = o_add(t43, a9); a9 = o_sub(t43, a9); }
    { uint64_t t44 = a14; a14 = o_add(t44, a19); a19 = o_sub(t44, a19); }
    { uint64_t t45 = a12; a12 = o_add(t45, a2); a2 = o_sub(t45, a2); }
    { uint64_t t46 = a17; a17 = o_add(t46, a7); a7 = o_sub(t46, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t47 = a12; a12 = o_add(t47, a17); a17 = o_sub(t47, a17); }
    { uint64_t t48 = a2; a2 = o_add(t48, a7); a7 = o_sub(t48, a7); }
    { uint64_t t49 = a16; a16 = o_add(t49, a6); a6 = o_sub(t49, a6); }
    { uint64_t t50 = a1; a1 = o_add(t50, a11); a11 = o_sub(t50, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t51 = a16; a16 = o_add(t51, a1); a1 = o_sub(t51, a1); }
    { uint64_t t52 = a6; a6 = o_add(t52, a11); a11 = o_sub(t52, a11); }
    { uint64_t t53 = a8; a8 = o_add(t53, a18); a18 = o_sub(t53, a18); }
    { uint64_t t54 = a13; a13 = o_add(t54, a3); a3 = o_sub(t54, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t55 = a8; a8 = o_add(t55, a13); a13 = o_sub(t55, a13); }
    { uint64_t t56 = a18; a18 = o_add(t56, a3); a3 = o_sub(t56, a3); }
    v[0] = a0;
    v[1] = a14;
    v[2] = a17;
    v[3] = a11;
    v[4] = a8;
    v[5] = a10;
    v[6] = a9;
    v[7] = a7;
    v[8] = a16;
    v[9] = a18;
    v[10] = a5;
    v[11] = a19;
    v[12] = a12;
    v[13] = a6;
    v[14] = a13;
    v[15] = a15;
    v[16] = a4;
    v[17] = a2;
    v[18] = a1;
    v[19] = a3;
}

static void o_ntt_24(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23];
    { uint64_t t1 = a0; a0 = o_add(t1, a12); a12 = o_sub(t1, a12); }
    { uint64_t t2 = a6; a6 = o_add(t2, a18); a18 = o_sub(t2, a18); }
    a18 = o_shift(a18, 48);
    { uint64_t t3 = a0; a0 = o_add(t3, a6); a6 = o_sub(t3, a6); }
    { uint64_t t4 = a12; a12 = o_add(t4, a18); a18 = o_sub(t4, a18); }
    { uint64_t t5 = a1; a1 = o_add(t5, a13); a13 = o_sub(t5, a13); }
    { uint64_t t6 = a7; a7 = o_add(t6, a19); a19 = o_sub(t6, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t7 = a1; a1 = o_add(t7, a7); a7 = o_sub(t7, a7); }
    { uint64_t t8 = a13; a13 = o_add(t8, a19); a19 = o_sub(t8, a19); }
    { uint64_t t9 = a2; a2 = o_add(t9, a14); a14 = o_sub(t9, a14); }
    { uint64_t t10 = a8; a8 = o_add(t10, a20); a20 = o_sub(t10, a20); }
    a20 = o_shift(a20, 48);
    { uint64_t t11 = a2; a2 = o_add(t11, a8); a8 = o_sub(t11, a8); }
    { uint64_t t12 = a14; a14 = o_add(t12, a20); a20 = o_sub(t12, a20); }
    { uint64_t t13 = a3; a3 = o_add(t13, a15); a15 = o_sub(t13, a15); }
    { uint64_t t14 = a9; a9 = o_add(t14, a21); a21 = o_sub(t14, a21); }
    a21 = o_shift(a21, 48);
    { uint64_t t15 = a3; a3 = o_add(t15, a9); a9 = o_sub(t15, a9); }
    { uint64_t t16 = a15; a15 = o_add(t16, a21); a21 = o_sub(t16, a21); }
    { uint64_t t17 = a4; a4 = o_add(t17, a16); a16 = o_sub(t17, a16); }
    { uint64_t t18 = a10; a10 = o_add(t18, a22); a22 = o_sub(t18, a22); }
    a22 = o_shift(a22, 48);
    { uint64_t t19 = a4; a4 = o_add(t19, a10); a10 = o_sub(t19, a10); }
    { uint64_t t20 = a16; a16 = o_add(t20, a22); a22 = o_sub(t20, a22); }
    { uint64_t t21 = a5; a5 = o_add(t21, a17); a17 = o_sub(t21, a17); }
    { uint64_t t22 = a11; a11 = o_add(t22, a23); a23 = o_sub(t22, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t23 = a5; a5 = o_add(t23, a11); a11 = o_sub(t23, a11); }
    { uint64_t t24 = a17; a17 = o_add(t24, a23); a23 = o_sub(t24, a23); }
    a13 = o_shift(a13, 8);
    a7 = o_shift(a7, 16);
    a19 = o_shift(a19, 24);
    a14 = o_shift(a14, 16);
    a8 = o_shift(a8, 32);
    a20 = o_shift(a20, 48);
    a15 = o_shift(a15, 24);
    a9 = o_shift(a9, 48);
    a21 = o_shift(a21, 72);
    a16 = o_shift(a16, 32);
    a10 = o_shift(a10, 64);
    a22 = o_neg(a22);
    a17 = o_shift(a17, 40);
    a11 = o_shift(a11, 80);
    a23 = o_neg(o_shift(a23, 24));
    { uint64_t t25 = a0, t26 = a2, t27 = a4;
      a0 = o_add(o_add(t25, t26), t27);
      a2 = o_sub(o_add(t25, o_shift(t26, 64)), o_shift(t27, 32));
      a4 = o_add(o_sub(t25, o_shift(t26, 32)), o_shift(t27, 64)); }
    { uint64_t t28 = a3, t29 = a5, t30 = a1;
      a3 = o_add(o_add(t28, t29), t30);
      a5 = o_sub(o_add(t28, o_shift(t29, 64)), o_shift(t30, 32));
      a1 = o_add(o_sub(t28, o_shift(t29, 32)), o_shift(t30, 64)); }
    { uint64_t t31 = a0; a0 = o_add(t31, a3); a3 = o_sub(t31, a3); }
    { uint64_t t32 = a2; a2 = o_add(t32, a5); a5 = o_sub(t32, a5); }
    { uint64_t t33 = a4; a4 = o_add(t33, a1); a1 = o_sub(t33, a1); }
    { uint64_t t34 = a12, t35 = a14, t36 = a16;
      a12 = o_add(o_add(t34, t35), t36);
      a14 = o_sub(o_add(t34, o_shift(t35, 64)), o_shift(t36, 32));
      a16 = o_add(o_sub(t34, o_shift(t35, 32)), o_shift(t36, 64)); }
    { uint64_t t37 = a15, t38 = a17, t39 = a13;
      a15 = o_add(o_add(t37, t38), t39);
      a17 = o_sub(o_add(t37, o_shift(t38, 64)), o_shift(t39, 32));
      a13 = o_add(o_sub(t37, o_shift(t38, 32)), o_shift(t39, 64)); }
    { uint64_t t40 = a12; a12 = o_add(t40, a15); a15 = o_sub(t40, a15); }
    { uint64_t t41 = a14; a14 = o_add(t41, a17); a17 = o_sub(t41, a17); }
    { uint64_t t42 = a16; a16 = o_add(t42, a13); a13 = o_sub(t42, a13); }
    { uint64_t t43 = a6, t44 = a8, t45 = a10;
      a6 = o_add(o_add(t43, t44), t45);
      a8 = o_sub(o_add(t43, o_shift(t44, 64)), o_shift(t45, 32));
      a10 = o_add(o_sub(t43, o_shift(t44, 32)), o_shift(t45, 64)); }
    { uint64_t t46 = a9, t47 = a11, t48 = a7;
      a9 = o_add(o_add(t46, t47), t48);
      a11 = o_sub(o_add(t46, o_shift(t47, 64)), o_shift(t48, 32));
      a7 = o_add(o_sub(t46, o_shift(t47, 32)), o_shift(t48, 64)); }
    { uint64_t t49 = a6; a6 = o_add(t49, a9); a9 = o_sub(t49, a9); }
    { uint64_t t50 = a8; a8 = o_add(t50, a11); a11 = o_sub(t50, a11); }
    { uint64_t t51 = a10; a10 = o_add(t51, a7); a7 = o_sub(t51, a7); }
    { uint64_t t52 = a18, t53 = a20, t54 = a22;
      a18 = o_add(o_add(t52, t53), t54);
      a20 = o_sub(o_add(t52, o_shift(t53, 64)), o_shift(t54, 32));
      a22 = o_add(o_sub(t52, o_shift(t53, 32)), o_shift(t54, 64)); }
    { uint64_t t55 = a21, t56 = a23, t57 = a19;
      a21 = o_add(o_add(t55, t56), t57);
      a23 = o_sub(o_add(t55, o_shift(t56, 64)), o_shift(t57, 32));
      a19 = o_add(o_sub(t55, o_shift(t56, 32)), o_shift(t57, 64)); }
    { uint64_t t58 = a18; a18 = o_add(t58, a21); a21 = o_sub(t58, a21); }
    { uint64_t t59 = a20; a20 = o_add(t59, a23); a23 = o_sub(t59, a23); }
    { uint64_t t60 = a22; a22 = o_add(t60, a19); a19 = o_sub(t60, a19); }
    v[0] = a0;
    v[1] = a12;
    v[2] = a6;
    v[3] = a18;
    v[4] = a5;
    v[5] = a17;
    v[6] = a11;
    v[7] = a23;
    v[8] = a4;
    v[9] = a16;
    v[10] = a10;
    v[11] = a22;
    v[12] = a3;
    v[13] = a15;
    v[14] = a9;
    v[15] = a21;
    v[16] = a2;
    v[17] = a14;
    v[18] = a8;
    v[19] = a20;
    v[20] = a1;
    v[21] = a13;
    v[22] = a7;
    v[23] = a19;
}

static void o_ntt_30(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29];
    { uint64_t t1 = a0, t2 = a10, t3 = a20;
      a0 = o_add(o_add(t1, t2), t3);
      a10 = o_sub(o_add(t1, o_shift(t2, 64)), o_shift(t3, 32));
      a20 = o_add(o_sub(t1, o_shift(t2, 32)), o_shift(t3, 64)); }
    { uint64_t t4 = a15, t5 = a25, t6 = a5;
      a15 = o_add(o_add(t4, t5), t6);
      a25 = o_sub(o_add(t4, o_shift(t5, 64)), o_shift(t6, 32));
      a5 = o_add(o_sub(t4, o_shift(t5, 32)), o_shift(t6, 64)); }
    { uint64_t t7 = a0; a0 = o_add(t7, a15); a15 = o_sub(t7, a15); }
    { uint64_t t8 = a10; a10 = o_add(t8, a25); a25 = o_sub(t8, a25); }
    { uint64_t t9 = a20; a20 = o_add(t9, a5); a5 = o_sub(t9, a5); }
    { uint64_t t10 = a6, t11 = a16, t12 = a26;
      a6 = o_add(o_add(t10, t11), t12);
      a16 = o_sub(o_add(t10, o_shift(t11, 64)), o_shift(t12, 32));
      a26 = o_add(o_sub(t10, o_shift(t11, 32)), o_shift(t12, 64)); }
    { uint64_t t13 = a21, t14 = a1, t15 = a11;
      a21 = o_add(o_add(t13, t14), t15);
      a1 = o_sub(o_add(t13, o_shift(t14, 64)), o_shift(t15, 32));
      a11 = o_add(o_sub(t13, o_shift(t14, 32)), o_shift(t15, 64)); }
    { uint64_t t16 = a6; a6 = o_add(t16, a21); a21 = o_sub(t16, a21); }
    { uint64_t t17 = a16; a16 = o_add(t17, a1); a1 = o_sub(t17, a1); }
    { uint64_t t18 = a26; a26 = o_add(t18, a11); a11 = o_sub(t18, a11); }
    { uint64_t t19 = a12, t20 = a22, t21 = a2;
      a12 = o_add(o_add(t19, t20), t21);
      a22 = o_sub(o_add(t19, o_shift(t20, 64)), o_shift(t21, 32));
      a2 = o_add(o_sub(t19, o_shift(t20, 32)), o_shift(t21, 64)); }
    { uint64_t t22 = a27, t23 = a7, t24 = a17;
      a27 = o_add(o_add(t22, t23), t24);
      a7 = o_sub(o_add(t22, o_shift(t23, 64)), o_shift(t24, 32));
      a17 = o_add(o_sub(t22, o_shift(t23, 32)), o_shift(t24, 64)); }
    { uint64_t t25 = a12; a12 = o_add(t25, a27); a27 = o_sub(t25, a27); }
    { uint64_t t26 = a22; a22 = o_add(t26, a7); a7 = o_sub(t26, a7); }
    { uint64_t t27 = a2; a2 = o_add(t27, a17); a17 = o_sub(t27, a17); }
    { uint64_t t28 = a18, t29 = a28, t30 = a8;
      a18 = o_add(o_add(t28, t29), t30);
      a28 = o_sub(o_add(t28, o_shift(t29, 64)), o_shift(t30, 32));
      a8 = o_add(o_sub(t28, o_shift(t29, 32)), o_shift(t30, 64)); }
    { uint64_t t31 = a3, t32 = a13, t33 = a23;
      a3 = o_add(o_add(t31, t32), t33);
      a13 = o_sub(o_add(t31, o_shift(t32, 64)), o_shift(t33, 32));
      a23 = o_add(o_sub(t31, o_shift(t32, 32)), o_shift(t33, 64)); }
    { uint64_t t34 = a18; a18 = o_add(t34, a3); a3 = o_sub(t34, a3); }
    { uint64_t t35 = a28; a28 = o_add(t35, a13); a13 = o_sub(t35, a13); }
    { uint64_t t36 = a8; a8 = o_add(t36, a23); a23 = o_sub(t36, a23); }
    { uint64_t t37 = a24, t38 = a4, t39 = a14;
      a24 = o_add(o_add(t37, t38), t39);
      a4 = o_sub(o_add(t37, o_shift(t38, 64)), o_shift(t39, 32));
      a14 = o_add(o_sub(t37, o_shift(t38, 32)), o_shift(t39, 64)); }
    { uint64_t t40 = a9, t41 = a19, t42 = a29;
      a9 = o_add(o_add(t40, t41), t42);
      a19 = o_sub(o_add(t40, o_shift(t41, 64)), o_shift(t42, 32));
      a29 = o_add(o_sub(t40, o_shift(t41, 32)), o_shift(t42, 64)); }
    { uint64_t t43 = a24; a24 = o_add(t43, a9); a9 = o_sub(t43, a9); }
    { uint64_t t44 = a4; a4 = o_add(t44, a19); a19 = o_sub(t44, a19); }
    { uint64_t t45 = a14; a14 = o_add(t45, a29); a29 = o_sub(t45, a29); }
    { uint64_t t46 = a6; a6 = o_add(t46, a24); a24 = o_sub(t46, a24); }
    { uint64_t t47 = a18; a18 = o_add(t47, a12); a12 = o_sub(t47, a12); }
    a12 = o_shift(a12, 48);
    { uint64_t t48 = a6; a6 = o_add(t48, a18); a18 = o_sub(t48, a18); }
    { uint64_t t49 = a24; a24 = o_add(t49, a12); a12 = o_sub(t49, a12); }
    uint64_t t50 = a0;
    a0 = o_add(a0, a6);
    a6 = o_mul(a6, 4611686017353646080ULL);
    a24 = o_mul(a24, 16181989089180173841ULL);
    a18 = o_mul(a18, 5818851782451133869ULL);
    a12 = o_mul(a12, 11322249509082494407ULL);
    a6 = o_add(a6, t50);
    { uint64_t t51 = a6; a6 = o_add(t51, a18); a18 = o_sub(t51, a18); }
    { uint64_t t52 = a12; a12 = o_add(t52, a24); a24 = o_sub(t52, a24); }
    a24 = o_shift(a24, 48);
    { uint64_t t53 = a6; a6 = o_add(t53, a12); a12 = o_sub(t53, a12); }
    { uint64_t t54 = a18; a18 = o_add(t54, a24); a24 = o_sub(t54, a24); }
    { uint64_t t55 = a1; a1 = o_add(t55, a19); a19 = o_sub(t55, a19); }
    { uint64_t t56 = a13; a13 = o_add(t56, a7); a7 = o_sub(t56, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t57 = a1; a1 = o_add(t57, a13); a13 = o_sub(t57, a13); }
    { uint64_t t58 = a19; a19 = o_add(t58, a7); a7 = o_sub(t58, a7); }
    uint64_t t59 = a25;
    a25 = o_add(a25, a1);
    a1 = o_mul(a1, 4611686017353646080ULL);
    a19 = o_mul(a19, 16181989089180173841ULL);
    a13 = o_mul(a13, 5818851782451133869ULL);
    a7 = o_mul(a7, 11322249509082494407ULL);
    a1 = o_add(a1, t59);
    { uint64_t t60 = a1; a1 = o_add(t60, a13); a13 = o_sub(t60, a13); }
    { uint64_t t61 = a7; a7 = o_add(t61, a19); a19 = o_sub(t61, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t62 = a1; a1 = o_add(t62, a7); a7 = o_sub(t62, a7); }
    { uint64_t t63 = a13; a13 = o_add(t63, a19); a19 = o_sub(t63, a19); }
    { uint64_t t64 = a26; a26 = o_add(t64, a14); a14 = o_sub(t64, a14); }
    { uint64_t t65 = a8; a8 = o_add(t65, a2); a2 = o_sub(t65, a2); }
    a2 = o_shift(a2, 48);
    { uint64_t t66 = a26; a26 = o_add(t66, a8); a8 = o_sub(t66, a8); }
    { uint64_t t67 = a14; a14 = o_add(t67, a2); a2 = o_sub(t67, a2); }
    uint64_t t68 = a20;
    a20 = o_add(a20, a26);
    a26 = o_mul(a26, 4611686017353646080ULL);
    a14 = o_mul(a14, 16181989089180173841ULL);
    a8 = o_mul(a8, 5818851782451133869ULL);
    a2 = o_mul(a2, 11322249509082494407ULL);
    a26 = o_add(a26, t68);
    { uint64_t t69 = a26; a26 = o_add(t69, a8); a8 = o_sub(t69, a8); }
    { uint64_t t70 = a2; a2 = o_add(t70, a14); a14 = o_sub(t70, a14); }
    a14 = o_shift(a14, 48);
    { uint64_t t71 = a26; a26 = o_add(t71, a2); a2 = o_sub(t71, a2); }
    { uint64_t t72 = a8; a8 = o_add(t72, a14); a14 = o_sub(t72, a14); }
    { uint64_t t73 = a21; a21 = o_add(t73, a9); a9 = o_sub(t73, a9); }
    { uint64_t t74 = a3; a3 = o_add(t74, a27); a27 = o_sub(t74, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t75 = a21; a21 = o_add(t75, a3); a3 = o_sub(t75, a3); }
    { uint64_t t76 = a9; a9 = o_add(t76, a27); a27 = o_sub(t76, a27); }
    uint64_t t77 = a15;
    a15 = o_add(a15, a21);
    a21 = o_mul(a21, 4611686017353646080ULL);
    a9 = o_mul(a9, 16181989089180173841ULL);
    a3 = o_mul(a3, 5818851782451133869ULL);
    a27 = o_mul(a27, 11322249509082494407ULL);
    a21 = o_add(a21, t77);
    { uint64_t t78 = a21; a21 = o_add(t78, a3); a3 = o_sub(t78, a3); }
    { uint64_t t79 = a27; a27 = o_add(t79, a9); a9 = o_sub(t79, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t80 = a21; a21 = o_add(t80, a27); a27 = o_sub(t80, a27); }
    { uint64_t t81 = a3; a3 = o_add(t81, a9); a9 = o_sub(t81, a9); }
    { uint64_t t82 = a16; a16 = o_add(t82, a4); a4 = o_sub(t82, a4); }
    { uint64_t t83 = a28; a28 = o_add(t83, a22); a22 = o_sub(t83, a22); }
    a22 = o_shift(a22, 48);
    { uint64_t t84 = a16; a16 = o_add(t84, a28); a28 = o_sub(t84, a28); }
    { uint64_t t85 = a4; a4 = o_add(t85, a22); a22 = o_sub(t85, a22); }
    uint64_t t86 = a10;
    a10 = o_add(a10, a16);
    a16 = o_mul(a16, 4611686017353646080ULL);
    a4 = o_mul(a4, 16181989089180173841ULL);
    a28 = o_mul(a28, 5818851782451133869ULL);
    a22 = o_mul(a22, 11322249509082494407ULL);
    a16 = o_add(a16, t86);
    { uint64_t t87 = a16; a16 = o_add(t87, a28); a28 = o_sub(t87, a28); }
    { uint64_t t88 = a22; a22 = o_add(t88, a4); a4 = o_sub(t88, a4); }
    a4 = o_shift(a4, 48);
    { uint64_t t89 = a16; a16 = o_add(t89, a22); a22 = o_sub(t89, a22); }
    { uint64_t t90 = a28; a28 = o_add(t90, a4); a4 = o_sub(t90, a4); }
    { uint64_t t91 = a11; a11 = o_add(t91, a29); a29 = o_sub(t91, a29); }
    { uint64_t t92 = a23; a23 = o_add(t92, a17); a17 = o_sub(t92, a17); }
    a17 = o_shift(a17, 48);
    { uint64_t t93 = a11; a11 = o_add(t93, a23); a23 = o_sub(t93, a23); }
    { uint64_t t94 = a29; a29 = o_add(t94, a17); a17 = o_sub(t94, a17); }
    uint64_t t95 = a5;
    a5 = o_add(a5, a11);
    a11 = o_mul(a11, 4611686017353646080ULL);
    a29 = o_mul(a29, 16181989089180173841ULL);
    a23 = o_mul(a23, 5818851782451133869ULL);
    a17 = o_mul(a17, 11322249509082494407ULL);
    a11 = o_add(a11, t95);
    { uint64_t t96 = a11; a11 = o_add(t96, a23); a23 = o_sub(t96, a23); }
    { uint64_t t97 = a17; a17 = o_add(t97, a29); a29 = o_sub(t97, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t98 = a11; a11 = o_add(t98, a17); a17 = o_sub(t98, a17); }
    { uint64_t t99 = a23; a23 = o_add(t99, a29); a29 = o_sub(t99, a29); }
    v[0] = a0;
    v[1] = a1;
    v[2] = a8;
    v[3] = a9;
    v[4] = a22;
    v[5] = a5;
    v[6] = a6;
    v[7] = a13;
    v[8] = a14;
    v[9] = a27;
    v[10] = a10;
    v[11] = a11;
    v[12] = a18;
    v[13] = a19;
    v[14] = a2;
    v[15] = a15;
    v[16] = a16;
    v[17] = a23;
    v[18] = a24;
    v[19] = a7;
    v[20] = a20;
    v[21] = a21;
    v[22] = a28;
    v[23] = a29;
    v[24] = a12;
    v[25] = a25;
    v[26] = a26;
    v[27] = a3;
    v[28] = a4;
    v[29] = a17;
}

static void o_ntt_32(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31];
    { uint64_t t1 = a0; a0 = o_add(t1, a16); a16 = o_sub(t1, a16); }
    { uint64_t t2 = a8; a8 = o_add(t2, a24); a24 = o_sub(t2, a24); }
    a24 = o_shift(a24, 48);
    { uint64_t t3 = a0; a0 = o_add(t3, a8); a8 = o_sub(t3, a8); }
    { uint64_t t4 = a16; a16 = o_add(t4, a24); a24 = o_sub(t4, a24); }
    { uint64_t t5 = a1; a1 = o_add(t5, a17); a17 = o_sub(t5, a17); }
    { uint64_t t6 = a9; a9 = o_add(t6, a25); a25 = o_sub(t6, a25); }
    a25 = o_shift(a25, 48);
    { uint64_t t7 = a1; a1 = o_add(t7, a9); a9 = o_sub(t7, a9); }
    { uint64_t t8 = a17; a17 = o_add(t8, a25); a25 = o_sub(t8, a25); }
    { uint64_t t9 = a2; a2 = o_add(t9, a18); a18 = o_sub(t9, a18); }
    { uint64_t t10 = a10; a10 = o_add(t10, a26); a26 = o_sub(t10, a26); }
    a26 = o_shift(a26, 48);
    { uint64_t t11 = a2; a2 = o_add(t11, a10); a10 = o_sub(t11, a10); }
    { uint64_t t12 = a18; a18 = o_add(t12, a26); a26 = o_sub(t12, a26); }
    { uint64_t t13 = a3; a3 = o_add(t13, a19); a19 = o_sub(t13, a19); }
    { uint64_t t14 = a11; a11 = o_add(t14, a27); a27 = o_sub(t14, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t15 = a3; a3 = o_add(t15, a11); a11 = o_sub(t15, a11); }
    { uint64_t t16 = a19; a19 = o_add(t16, a27); a27 = o_sub(t16, a27); }
    { uint64_t t17 = a4; a4 = o_add(t17, a20); a20 = o_sub(t17, a20); }
    { uint64_t t18 = a12; a12 = o_add(t18, a28); a28 = o_sub(t18, a28); }
    a28 = o_shift(a28, 48);
    { uint64_t t19 = a4; a4 = o_add(t19, a12); a12 = o_sub(t19, a12); }
    { uint64_t t20 = a20; a20 = o_add(t20, a28); a28 = o_sub(t20, a28); }
    { uint64_t t21 = a5; a5 = o_add(t21, a21); a21 = o_sub(t21, a21); }
    { uint64_t t22 = a13; a13 = o_add(t22, a29); a29 = o_sub(t22, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t23 = a5; a5 = o_add(t23, a13); a13 = o_sub(t23, a13); }
    { uint64_t t24 = a21; a21 = o_add(t24, a29); a29 = o_sub(t24, a29); }
    { uint64_t t25 = a6; a6 = o_add(t25, a22); a22 = o_sub(t25, a22); }
    { uint64_t t26 = a14; a14 = o_add(t26, a30); a30 = o_sub(t26, a30); }
    a30 = o_shift(a30, 48);
    { uint64_t t27 = a6; a6 = o_add(t27, a14); a14 = o_sub(t27, a14); }
    { uint64_t t28 = a22; a22 = o_add(t28, a30); a30 = o_sub(t28, a30); }
    { uint64_t t29 = a7; a7 = o_add(t29, a23); a23 = o_sub(t29, a23); }
    { uint64_t t30 = a15; a15 = o_add(t30, a31); a31 = o_sub(t30, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t31 = a7; a7 = o_add(t31, a15); a15 = o_sub(t31, a15); }
    { uint64_t t32 = a23; a23 = o_add(t32, a31); a31 = o_sub(t32, a31); }
    a17 = o_shift(a17, 6);
    a9 = o_shift(a9, 12);
    a25 = o_shift(a25, 18);
    a18 = o_shift(a18, 12);
    a10 = o_shift(a10, 24);
    a26 = o_shift(a26, 36);
    a19 = o_shift(a19, 18);
    a11 = o_shift(a11, 36);
    a27 = o_shift(a27, 54);
    a20 = o_shift(a20, 24);
    a12 = o_shift(a12, 48);
    a28 = o_shift(a28, 72);
    a21 = o_shift(a21, 30);
    a13 = o_shift(a13, 60);
    a29 = o_shift(a29, 90);
    a22 = o_shift(a22, 36);
    a14 = o_shift(a14, 72);
    a30 = o_neg(o_shift(a30, 12));
    a23 = o_shift(a23, 42);
    a15 = o_shift(a15, 84);
    a31 = o_neg(o_shift(a31, 30));
    { uint64_t t33 = a0; a0 = o_add(t33, a4); a4 = o_sub(t33, a4); }
    { uint64_t t34 = a1; a1 = o_add(t34, a5); a5 = o_sub(t34, a5); }
    { uint64_t t35 = a2; a2 = o_add(t35, a6); a6 = o_sub(t35, a6); }
    { uint64_t t36 = a3; a3 = o_add(t36, a7); a7 = o_sub(t36, a7); }
    a5 = o_shift(a5, 24);
    a6 = o_shift(a6, 48);
    a7 = o_shift(a7, 72);
    { uint64_t t37 = a0; a0 = o_add(t37, a2); a2 = o_sub(t37, a2); }
    { uint64_t t38 = a1; a1 = o_add(t38, a3); a3 = o_sub(t38, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t39 = a0; a0 = o_add(t39, a1); a1 = o_sub(t39, a1); }
    { uint64_t t40 = a2; a2 = o_add(t40, a3); a3 = o_sub(t40, a3); }
    { uint64_t t41 = a4; a4 = o_add(t41, a6); a6 = o_sub(t41, a6); }
    { uint64_t t42 = a5; a5 = o_add(t42, a7); a7 = o_sub(t42, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t43 = a4; a4 = o_add(t43, a5); a5 = o_sub(t43, a5); }
    { uint64_t t44 = a6; a6 = o_add(t44, a7); a7 = o_sub(t44, a7); }
    { uint64_t t45 = a16; a16 = o_add(t45, a20); a20 = o_sub(t45, a20); }
    { uint64_t t46 = a17; a17 = o_add(t46, a21); a21 = o_sub(t46, a21); }
    { uint64_t t47 = a18; a18 = o_add(t47, a22); a22 = o_sub(t47, a22); }
    { uint64_t t48 = a19; a19 = o_add(t48, a23); a23 = o_sub(t48, a23); }
    a21 = o_shift(a21, 24);
    a22 = o_shift(a22, 48);
    a23 = o_shift(a23, 72);
    { uint64_t t49 = a16; a16 = o_add(t49, a18); a18 = o_sub(t49, a18); }
    { uint64_t t50 = a17; a17 = o_add(t50, a19); a19 = o_sub(t50, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t51 = a16; a16 = o_add(t51, a17); a17 = o_sub(t51, a17); }
    { uint64_t t52 = a18; a18 = o_add(t52, a19); a19 = o_sub(t52, a19); }
    { uint64_t t53 = a20; a20 = o_add(t53, a22); a22 = o_sub(t53, a22); }
    { uint64_t t54 = a21; a21 = o_add(t54, a23); a23 = o_sub(t54, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t55 = a20; a20 = o_add(t55, a21); a21 = o_sub(t55, a21); }
    { uint64_t t56 = a22; a22 = o_add(t56, a23); a23 = o_sub(t56, a23); }
    { uint64_t t57 = a8; a8 = o_add(t57, a12); a12 = o_sub(t57, a12); }
    { uint64_t t58 = a9; a9 = o_add(t58, a13); a13 = o_sub(t58, a13); }
    { uint64_t t59 = a10; a10 = o_add(t59, a14); a14 = o_sub(t59, a14); }
    { uint64_t t60 = a11; a11 = o_add(t60, a15); a15 = o_sub(t60, a15); }
    a13 = o_shift(a13, 24);
    a14 = o_shift(a14, 48);
    a15 = o_shift(a15, 72);
    { uint64_t t61 = a8; a8 = o_add(t61, a10); a10 = o_sub(t61, a10); }
    { uint64_t t62 = a9; a9 = o_add(t62, a11); a11 = o_sub(t62, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t63 = a8; a8 = o_add(t63, a9); a9 = o_sub(t63, a9); }
    { uint64_t t64 = a10; a10 = o_add(t64, a11); a11 = o_sub(t64, a11); }
    { uint64_t t65 = a12; a12 = o_add(t65, a14); a14 = o_sub(t65, a14); }
    { uint64_t t66 = a13; a13 = o_add(t66, a15); a15 = o_sub(t66, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t67 = a12; a12 = o_add(t67, a13); a13 = o_sub(t67, a13); }
    { uint64_t t68 = a14; a14 = o_add(t68, a15); a15 = o_sub(t68, a15); }
    { uint64_t t69 = a24; a24 = o_add(t69, a28); a28 = o_sub(t69, a28); }
    { uint64_t t70 = a25; a25 = o_add(t70, a29); a29 = o_sub(t70, a29); }
    { uint64_t t71 = a26; a26 = o_add(t71, a30); a30 = o_sub(t71, a30); }
    { uint64_t t72 = a27; a27 = o_add(t72, a31); a31 = o_sub(t72, a31); }
    a29 = o_shift(a29, 24);
    a30 = o_shift(a30, 48);
    a31 = o_shift(a31, 72);
    { uint64_t t73 = a24; a24 = o_add(t73, a26); a26 = o_sub(t73, a26); }
    { uint64_t t74 = a25; a25 = o_add(t74, a27); a27 = o_sub(t74, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t75 = a24; a24 = o_add(t75, a25); a25 = o_sub(t75, a25); }
    { uint64_t t76 = a26; a26 = o_add(t76, a27); a27 = o_sub(t76, a27); }
    { uint64_t t77 = a28; a28 = o_add(t77, a30); a30 = o_sub(t77, a30); }
    { uint64_t t78 = a29; a29 = o_add(t78, a31); a31 = o_sub(t78, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t79 = a28; a28 = o_add(t79, a29); a29 = o_sub(t79, a29); }
    { uint64_t t80 = a30; a30 = o_add(t80, a31); a31 = o_sub(t80, a31); }
    v[0] = a0;
    v[1] = a16;
    v[2] = a8;
    v[3] = a24;
    v[4] = a4;
    v[5] = a20;
    v[6] = a12;
    v[7] = a28;
    v[8] = a2;
    v[9] = a18;
    v[10] = a10;
    v[11] = a26;
    v[12] = a6;
    v[13] = a22;
    v[14] = a14;
    v[15] = a30;
    v[16] = a1;
    v[17] = a17;
    v[18] = a9;
    v[19] = a25;
    v[20] = a5;
    v[21] = a21;
    v[22] = a13;
    v[23] = a29;
    v[24] = a3;
    v[25] = a19;
    v[26] = a11;
    v[27] = a27;
    v[28] = a7;
    v[29] = a23;
    v[30] = a15;
    v[31] = a31;
}

static void o_ntt_34(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33];
    { uint64_t t1 = a2; a2 = o_add(t1, a32); a32 = o_sub(t1, a32); }
    { uint64_t t2 = a8; a8 = o_add(t2, a26); a26 = o_sub(t2, a26); }
    a26 = o_shift(a26, 48);
    { uint64_t t3 = a2; a2 = o_add(t3, a8); a8 = o_sub(t3, a8); }
    { uint64_t t4 = a32; a32 = o_add(t4, a26); a26 = o_sub(t4, a26); }
    { uint64_t t5 = a12; a12 = o_add(t5, a22); a22 = o_sub(t5, a22); }
    { uint64_t t6 = a14; a14 = o_add(t6, a20); a20 = o_sub(t6, a20); }
    a20 = o_shift(a20, 48);
    { uint64_t t7 = a12; a12 = o_add(t7, a14); a14 = o_sub(t7, a14); }
    { uint64_t t8 = a22; a22 = o_add(t8, a20); a20 = o_sub(t8, a20); }
    { uint64_t t9 = a4; a4 = o_add(t9, a30); a30 = o_sub(t9, a30); }
    { uint64_t t10 = a16; a16 = o_add(t10, a18); a18 = o_sub(t10, a18); }
    a18 = o_shift(a18, 48);
    { uint64_t t11 = a4; a4 = o_add(t11, a16); a16 = o_sub(t11, a16); }
    { uint64_t t12 = a30; a30 = o_add(t12, a18); a18 = o_sub(t12, a18); }
    { uint64_t t13 = a24; a24 = o_add(t13, a10); a10 = o_sub(t13, a10); }
    { uint64_t t14 = a28; a28 = o_add(t14, a6); a6 = o_sub(t14, a6); }
    a6 = o_shift(a6, 48);
    { uint64_t t15 = a24; a24 = o_add(t15, a28); a28 = o_sub(t15, a28); }
    { uint64_t t16 = a10; a10 = o_add(t16, a6); a6 = o_sub(t16, a6); }
    a22 = o_shift(a22, 12);
    a14 = o_shift(a14, 24);
    a20 = o_shift(a20, 36);
    a30 = o_shift(a30, 24);
    a16 = o_shift(a16, 48);
    a18 = o_shift(a18, 72);
    a10 = o_shift(a10, 36);
    a28 = o_shift(a28, 72);
    a6 = o_neg(o_shift(a6, 12));
    { uint64_t t17 = a2; a2 = o_add(t17, a4); a4 = o_sub(t17, a4); }
    { uint64_t t18 = a12; a12 = o_add(t18, a24); a24 = o_sub(t18, a24); }
    a24 = o_shift(a24, 48);
    { uint64_t t19 = a2; a2 = o_add(t19, a12); a12 = o_sub(t19, a12); }
    { uint64_t t20 = a4; a4 = o_add(t20, a24); a24 = o_sub(t20, a24); }
    { uint64_t t21 = a32; a32 = o_add(t21, a30); a30 = o_sub(t21, a30); }
    { uint64_t t22 = a22; a22 = o_add(t22, a10); a10 = o_sub(t22, a10); }
    a10 = o_shift(a10, 48);
    { uint64_t t23 = a32; a32 = o_add(t23, a22); a22 = o_sub(t23, a22); }
    { uint64_t t24 = a30; a30 = o_add(t24, a10); a10 = o_sub(t24, a10); }
    { uint64_t t25 = a8; a8 = o_add(t25, a16); a16 = o_sub(t25, a16); }
    { uint64_t t26 = a14; a14 = o_add(t26, a28); a28 = o_sub(t26, a28); }
    a28 = o_shift(a28, 48);
    { uint64_t t27 = a8; a8 = o_add(t27, a14); a14 = o_sub(t27, a14); }
    { uint64_t t28 = a16; a16 = o_add(t28, a28); a28 = o_sub(t28, a28); }
    { uint64_t t29 = a26; a26 = o_add(t29, a18); a18 = o_sub(t29, a18); }
    { uint64_t t30 = a20; a20 = o_add(t30, a6); a6 = o_sub(t30, a6); }
    a6 = o_shift(a6, 48);
    { uint64_t t31 = a26; a26 = o_add(t31, a20); a20 = o_sub(t31, a20); }
    { uint64_t t32 = a18; a18 = o_add(t32, a6); a6 = o_sub(t32, a6); }
    uint64_t t33 = a0;
    a0 = o_add(a0, a2);
    a2 = o_mul(a2, 1152921504338411520ULL);
    a32 = o_mul(a32, 6259776822214049175ULL);
    a8 = o_mul(a8, 9380094172986290191ULL);
    a26 = o_mul(a26, 891943630314919127ULL);
    a4 = o_mul(a4, 17228171707553225791ULL);
    a30 = o_mul(a30, 12855743360534130886ULL);
    a16 = o_mul(a16, 6167687396920564837ULL);
    a18 = o_mul(a18, 17201834061724655524ULL);
    a12 = o_mul(a12, 15308299771656910737ULL);
    a22 = o_mul(a22, 18186005861103657533ULL);
    a14 = o_mul(a14, 53595491891823545ULL);
    a20 = o_mul(a20, 1906638201581172103ULL);
    a24 = o_mul(a24, 18303651001328874822ULL);
    a10 = o_mul(a10, 3077466521755967626ULL);
    a28 = o_mul(a28, 12423593102987598328ULL);
    a6 = o_mul(a6, 18361513053649472048ULL);
    a2 = o_add(a2, t33);
    { uint64_t t34 = a2; a2 = o_add(t34, a12); a12 = o_sub(t34, a12); }
    { uint64_t t35 = a24; a24 = o_add(t35, a4); a4 = o_sub(t35, a4); }
    a4 = o_shift(a4, 48);
    { uint64_t t36 = a2; a2 = o_add(t36, a24); a24 = o_sub(t36, a24); }
    { uint64_t t37 = a12; a12 = o_add(t37, a4); a4 = o_sub(t37, a4); }
    { uint64_t t38 = a6; a6 = o_add(t38, a18); a18 = o_sub(t38, a18); }
    { uint64_t t39 = a20; a20 = o_add(t39, a26); a26 = o_sub(t39, a26); }
    a26 = o_shift(a26, 48);
    { uint64_t t40 = a6; a6 = o_add(t40, a20); a20 = o_sub(t40, a20); }
    { uint64_t t41 = a18; a18 = o_add(t41, a26); a26 = o_sub(t41, a26); }
    { uint64_t t42 = a28; a28 = o_add(t42, a16); a16 = o_sub(t42, a16); }
    { uint64_t t43 = a14; a14 = o_add(t43, a8); a8 = o_sub(t43, a8); }
    a8 = o_shift(a8, 48);
    { uint64_t t44 = a28; a28 = o_add(t44, a14); a14 = o_sub(t44, a14); }
    { uint64_t t45 = a16; a16 = o_add(t45, a8); a8 = o_sub(t45, a8); }
    { uint64_t t46 = a10; a10 = o_add(t46, a30); a30 = o_sub(t46, a30); }
    { uint64_t t47 = a22; a22 = o_add(t47, a32); a32 = o_sub(t47, a32); }
    a32 = o_shift(a32, 48);
    { uint64_t t48 = a10; a10 = o_add(t48, a22); a22 = o_sub(t48, a22); }
    { uint64_t t49 = a30; a30 = o_add(t49, a32); a32 = o_sub(t49, a32); }
    a18 = o_shift(a18, 12);
    a20 = o_shift(a20, 24);
    a26 = o_shift(a26, 36);
    a16 = o_shift(a16, 24);
    a14 = o_shift(a14, 48);
    a8 = o_shift(a8, 72);
    a30 = o_shift(a30, 36);
    a22 = o_shift(a22, 72);
    a32 = o_neg(o_shift(a32, 12));
    { uint64_t t50 = a2; a2 = o_add(t50, a28); a28 = o_sub(t50, a28); }
    { uint64_t t51 = a6; a6 = o_add(t51, a10); a10 = o_sub(t51, a10); }
    a10 = o_shift(a10, 48);
    { uint64_t t52 = a2; a2 = o_add(t52, a6); a6 = o_sub(t52, a6); }
    { uint64_t t53 = a28; a28 = o_add(t53, a10); a10 = o_sub(t53, a10); }
    { uint64_t t54 = a12; a12 = o_add(t54, a16); a16 = o_sub(t54, a16); }
    { uint64_t t55 = a18; a18 = o_add(t55, a30); a30 = o_sub(t55, a30); }
    a30 = o_shift(a30, 48);
    { uint64_t t56 = a12; a12 = o_add(t56, a18); a18 = o_sub(t56, a18); }
    { uint64_t t57 = a16; a16 = o_add(t57, a30); a30 = o_sub(t57, a30); }
    { uint64_t t58 = a24; a24 = o_add(t58, a14); a14 = o_sub(t58, a14); }
    { uint64_t t59 = a20; a20 = o_add(t59, a22); a22 = o_sub(t59, a22); }
    a22 = o_shift(a22, 48);
    { uint64_t t60 = a24; a24 = o_add(t60, a20); a20 = o_sub(t60, a20); }
    { uint64_t t61 = a14; a14 = o_add(t61, a22); a22 = o_sub(t61, a22); }
    { uint64_t t62 = a4; a4 = o_add(t62, a8); a8 = o_sub(t62, a8); }
    { uint64_t t63 = a26; a26 = o_add(t63, a32); a32 = o_sub(t63, a32); }
    a32 = o_shift(a32, 48);
    { uint64_t t64 = a4; a4 = o_add(t64, a26); a26 = o_sub(t64, a26); }
    { uint64_t t65 = a8; a8 = o_add(t65, a32); a32 = o_sub(t65, a32); }
    { uint64_t t66 = a19; a19 = o_add(t66, a15); a15 = o_sub(t66, a15); }
    { uint64_t t67 = a25; a25 = o_add(t67, a9); a9 = o_sub(t67, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t68 = a19; a19 = o_add(t68, a25); a25 = o_sub(t68, a25); }
    { uint64_t t69 = a15; a15 = o_add(t69, a9); a9 = o_sub(t69, a9); }
    { uint64_t t70 = a29; a29 = o_add(t70, a5); a5 = o_sub(t70, a5); }
    { uint64_t t71 = a31; a31 = o_add(t71, a3); a3 = o_sub(t71, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t72 = a29; a29 = o_add(t72, a31); a31 = o_sub(t72, a31); }
    { uint64_t t73 = a5; a5 = o_add(t73, a3); a3 = o_sub(t73, a3); }
    { uint64_t t74 = a21; a21 = o_add(t74, a13); a13 = o_sub(t74, a13); }
    { uint64_t t75 = a33; a33 = o_add(t75, a1); a1 = o_sub(t75, a1); }
    a1 = o_shift(a1, 48);
    { uint64_t t76 = a21; a21 = o_add(t76, a33); a33 = o_sub(t76, a33); }
    { uint64_t t77 = a13; a13 = o_add(t77, a1); a1 = o_sub(t77, a1); }
    { uint64_t t78 = a7; a7 = o_add(t78, a27); a27 = o_sub(t78, a27); }
    { uint64_t t79 = a11; a11 = o_add(t79, a23); a23 = o_sub(t79, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t80 = a7; a7 = o_add(t80, a11); a11 = o_sub(t80, a11); }
    { uint64_t t81 = a27; a27 = o_add(t81, a23); a23 = o_sub(t81, a23); }
    a5 = o_shift(a5, 12);
    a31 = o_shift(a31, 24);
    a3 = o_shift(a3, 36);
    a13 = o_shift(a13, 24);
    a33 = o_shift(a33, 48);
    a1 = o_shift(a1, 72);
    a27 = o_shift(a27, 36);
    a11 = o_shift(a11, 72);
    a23 = o_neg(o_shift(a23, 12));
    { uint64_t t82 = a19; a19 = o_add(t82, a21); a21 = o_sub(t82, a21); }
    { uint64_t t83 = a29; a29 = o_add(t83, a7); a7 = o_sub(t83, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t84 = a19; a19 = o_add(t84, a29); a29 = o_sub(t84, a29); }
    { uint64_t t85 = a21; a21 = o_add(t85, a7); a7 = o_sub(t85, a7); }
    { uint64_t t86 = a15; a15 = o_add(t86, a13); a13 = o_sub(t86, a13); }
    { uint64_t t87 = a5; a5 = o_add(t87, a27); a27 = o_sub(t87, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t88 = a15; a15 = o_add(t88, a5); a5 = o_sub(t88, a5); }
    { uint64_t t89 = a13; a13 = o_add(t89, a27); a27 = o_sub(t89, a27); }
    { uint64_t t90 = a25; a25 = o_add(t90, a33); a33 = o_sub(t90, a33); }
    { uint64_t t91 = a31; a31 = o_add(t91, a11); a11 = o_sub(t91, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t92 = a25; a25 = o_add(t92, a31); a31 = o_sub(t92, a31); }
    { uint64_t t93 = a33; a33 = o_add(t93, a11); a11 = o_sub(t93, a11); }
    { uint64_t t94 = a9; a9 = o_add(t94, a1); a1 = o_sub(t94, a1); }
    { uint64_t t95 = a3; a3 = o_add(t95, a23); a23 = o_sub(t95, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t96 = a9; a9 = o_add(t96, a3); a3 = o_sub(t96, a3); }
    { uint64_t t97 = a1; a1 = o_add(t97, a23); a23 = o_sub(t97, a23); }
    uint64_t t98 = a17;
    a17 = o_add(a17, a19);
    a19 = o_mul(a19, 1152921504338411520ULL);
    a15 = o_mul(a15, 6259776822214049175ULL);
    a25 = o_mul(a25, 9380094172986290191ULL);
    a9 = o_mul(a9, 891943630314919127ULL);
    a21 = o_mul(a21, 17228171707553225791ULL);
    a13 = o_mul(a13, 12855743360534130886ULL);
    a33 = o_mul(a33, 6167687396920564837ULL);
    a1 = o_mul(a1, 17201834061724655524ULL);
    a29 = o_mul(a29, 15308299771656910737ULL);
    a5 = o_mul(a5, 18186005861103657533ULL);
    a31 = o_mul(a31, 53595491891823545ULL);
    a3 = o_mul(a3, 1906638201581172103ULL);
    a7 = o_mul(a7, 18303651001328874822ULL);
    a27 = o_mul(a27, 3077466521755967626ULL);
    a11 = o_mul(a11, 12423593102987598328ULL);
    a23 = o_mul(a23, 18361513053649472048ULL);
    a19 = o_add(a19, t98);
    { uint64_t t99 = a19; a19 = o_add(t99, a29); a29 = o_sub(t99, a29); }
    { uint64_t t100 = a7; a7 = o_add(t100, a21); a21 = o_sub(t100, a21); }
    a21 = o_shift(a21, 48);
    { uint64_t t101 = a19; a19 = o_add(t101, a7); a7 = o_sub(t101, a7); }
    { uint64_t t102 = a29; a29 = o_add(t102, a21); a21 = o_sub(t102, a21); }
    { uint64_t t103 = a23; a23 = o_add(t103, a1); a1 = o_sub(t103, a1); }
    { uint64_t t104 = a3; a3 = o_add(t104, a9); a9 = o_sub(t104, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t105 = a23; a23 = o_add(t105, a3); a3 = o_sub(t105, a3); }
    { uint64_t t106 = a1; a1 = o_add(t106, a9); a9 = o_sub(t106, a9); }
    { uint64_t t107 = a11; a11 = o_add(t107, a33); a33 = o_sub(t107, a33); }
    { uint64_t t108 = a31; a31 = o_add(t108, a25); a25 = o_sub(t108, a25); }
    a25 = o_shift(a25, 48);
    { uint64_t t109 = a11; a11 = o_add(t109, a31); a31 = o_sub(t109, a31); }
    { uint64_t t110 = a33; a33 = o_add(t110, a25); a25 = o_sub(t110, a25); }
    { uint64_t t111 = a27; a27 = o_add(t111, a13); a13 = o_sub(t111, a13); }
    { uint64_t t112 = a5; a5 = o_add(t112, a15); a15 = o_sub(t112, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t113 = a27; a27 = o_add(t113, a5); a5 = o_sub(t113, a5); }
    { uint64_t t114 = a13; a13 = o_add(t114, a15); a15 = o_sub(t114, a15); }
    a1 = o_shift(a1, 12);
    a3 = o_shift(a3, 24);
    a9 = o_shift(a9, 36);
    a33 = o_shift(a33, 24);
    a31 = o_shift(a31, 48);
    a25 = o_shift(a25, 72);
    a13 = o_shift(a13, 36);
    a5 = o_shift(a5, 72);
    a15 = o_neg(o_shift(a15, 12));
    { uint64_t t115 = a19; a19 = o_add(t115, a11); a11 = o_sub(t115, a11); }
    { uint64_t t116 = a23; a23 = o_add(t116, a27); a27 = o_sub(t116, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t117 = a19; a19 = o_add(t117, a23); a23 = o_sub(t117, a23); }
    { uint64_t t118 = a11; a11 = o_add(t118, a27); a27 = o_sub(t118, a27); }
    { uint64_t t119 = a29; a29 = o_add(t119, a33); a33 = o_sub(t119, a33); }
    { uint64_t t120 = a1; a1 = o_add(t120, a13); a13 = o_sub(t120, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t121 = a29; a29 = o_add(t121, a1); a1 = o_sub(t121, a1); }
    { uint64_t t122 = a33; a33 = o_add(t122, a13); a13 = o_sub(t122, a13); }
    { uint64_t t123 = a7; a7 = o_add(t123, a31); a31 = o_sub(t123, a31); }
    { uint64_t t124 = a3; a3 = o_add(t124, a5); a5 = o_sub(t124, a5); }
    a5 = o_shift(a5, 48);
    { uint64_t t125 = a7; a7 = o_add(t125, a3); a3 = o_sub(t125, a3); }
    { uint64_t t126 = a31; a31 = o_add(t126, a5); a5 = o_sub(t126, a5); }
    { uint64_t t127 = a21; a21 = o_add(t127, a25); a25 = o_sub(t127, a25); }
    { uint64_t t128 = a9; a9 = o_add(t128, a15); a15 = o_sub(t128, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t129 = a21; a21 = o_add(t129, a9); a9 = o_sub(t129, a9); }
    { uint64_t t130 = a25; a25 = o_add(t130, a15); a15 = o_sub(t130, a15); }
    { uint64_t t131 = a0; a0 = o_add(t131, a17); a17 = o_sub(t131, a17); }
    { uint64_t t132 = a2; a2 = o_add(t132, a19); a19 = o_sub(t132, a19); }
    { uint64_t t133 = a22; a22 = o_add(t133, a5); a5 = o_sub(t133, a5); }
    { uint64_t t134 = a12; a12 = o_add(t134, a29); a29 = o_sub(t134, a29); }
    { uint64_t t135 = a10; a10 = o_add(t135, a27); a27 = o_sub(t135, a27); }
    { uint64_t t136 = a16; a16 = o_add(t136, a33); a33 = o_sub(t136, a33); }
    { uint64_t t137 = a32; a32 = o_add(t137, a15); a15 = o_sub(t137, a15); }
    { uint64_t t138 = a26; a26 = o_add(t138, a9); a9 = o_sub(t138, a9); }
    { uint64_t t139 = a20; a20 = o_add(t139, a3); a3 = o_sub(t139, a3); }
    { uint64_t t140 = a24; a24 = o_add(t140, a7); a7 = o_sub(t140, a7); }
    { uint64_t t141 = a4; a4 = o_add(t141, a21); a21 = o_sub(t141, a21); }
    { uint64_t t142 = a8; a8 = o_add(t142, a25); a25 = o_sub(t142, a25); }
    { uint64_t t143 = a30; a30 = o_add(t143, a13); a13 = o_sub(t143, a13); }
    { uint64_t t144 = a28; a28 = o_add(t144, a11); a11 = o_sub(t144, a11); }
    { uint64_t t145 = a18; a18 = o_add(t145, a1); a1 = o_sub(t145, a1); }
    { uint64_t t146 = a14; a14 = o_add(t146, a31); a31 = o_sub(t146, a31); }
    { uint64_t t147 = a6; a6 = o_add(t147, a23); a23 = o_sub(t147, a23); }
    v[0] = a0;
    v[1] = a19;
    v[2] = a22;
    v[3] = a29;
    v[4] = a10;
    v[5] = a33;
    v[6] = a32;
    v[7] = a9;
    v[8] = a20;
    v[9] = a7;
    v[10] = a4;
    v[11] = a25;
    v[12] = a30;
    v[13] = a11;
    v[14] = a18;
    v[15] = a31;
    v[16] = a6;
    v[17] = a17;
    v[18] = a2;
    v[19] = a5;
    v[20] = a12;
    v[21] = a27;
    v[22] = a16;
    v[23] = a15;
    v[24] = a26;
    v[25] = a3;
    v[26] = a24;
    v[27] = a21;
    v[28] = a8;
    v[29] = a13;
    v[30] = a28;
    v[31] = a1;
    v[32] = a14;
    v[33] = a23;
}

static void o_ntt_40(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33], a34 = v[34], a35 = v[35], a36 = v[36], a37 = v[37], a38 = v[38], a39 = v[39];
    { uint64_t t1 = a0; a0 = o_add(t1, a20); a20 = o_sub(t1, a20); }
    { uint64_t t2 = a5; a5 = o_add(t2, a25); a25 = o_sub(t2, a25); }
    { uint64_t t3 = a10; a10 = o_add(t3, a30); a30 = o_sub(t3, a30); }
    { uint64_t t4 = a15; a15 = o_add(t4, a35); a35 = o_sub(t4, a35); }
    a25 = o_shift(a25, 24);
    a30 = o_shift(a30, 48);
    a35 = o_shift(a35, 72);
    { uint64_t t5 = a0; a0 = o_add(t5, a10); a10 = o_sub(t5, a10); }
    { uint64_t t6 = a5; a5 = o_add(t6, a15); a15 = o_sub(t6, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t7 = a0; a0 = o_add(t7, a5); a5 = o_sub(t7, a5); }
    { uint64_t t8 = a10; a10 = o_add(t8, a15); a15 = o_sub(t8, a15); }
    { uint64_t t9 = a20; a20 = o_add(t9, a30); a30 = o_sub(t9, a30); }
    { uint64_t t10 = a25; a25 = o_add(t10, a35); a35 = o_sub(t10, a35); }
    a35 = o_shift(a35, 48);
    { uint64_t t11 = a20; a20 = o_add(t11, a25); a25 = o_sub(t11, a25); }
    { uint64_t t12 = a30; a30 = o_add(t12, a35); a35 = o_sub(t12, a35); }
    { uint64_t t13 = a8; a8 = o_add(t13, a28); a28 = o_sub(t13, a28); }
    { uint64_t t14 = a13; a13 = o_add(t14, a33); a33 = o_sub(t14, a33); }
    { uint64_t t15 = a18; a18 = o_add(t15, a38); a38 = o_sub(t15, a38); }
    { uint64_t t16 = a23; a23 = o_add(t16, a3); a3 = o_sub(t16, a3); }
    a33 = o_shift(a33, 24);
    a38 = o_shift(a38, 48);
    a3 = o_shift(a3, 72);
    { uint64_t t17 = a8; a8 = o_add(t17, a18); a18 = o_sub(t17, a18); }
    { uint64_t t18 = a13; a13 = o_add(t18, a23); a23 = o_sub(t18, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t19 = a8; a8 = o_add(t19, a13); a13 = o_sub(t19, a13); }
    { uint64_t t20 = a18; a18 = o_add(t20, a23); a23 = o_sub(t20, a23); }
    { uint64_t t21 = a28; a28 = o_add(t21, a38); a38 = o_sub(t21, a38); }
    { uint64_t t22 = a33; a33 = o_add(t22, a3); a3 = o_sub(t22, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t23 = a28; a28 = o_add(t23, a33); a33 = o_sub(t23, a33); }
    { uint64_t t24 = a38; a38 = o_add(t24, a3); a3 = o_sub(t24, a3); }
    { uint64_t t25 = a16; a16 = o_add(t25, a36); a36 = o_sub(t25, a36); }
    { uint64_t t26 = a21; a21 = o_add(t26, a1); a1 = o_sub(t26, a1); }
    { uint64_t t27 = a26; a26 = o_add(t27, a6); a6 = o_sub(t27, a6); }
    { uint64_t t28 = a31; a31 = o_add(t28, a11); a11 = o_sub(t28, a11); }
    a1 = o_shift(a1, 24);
    a6 = o_shift(a6, 48);
    a11 = o_shift(a11, 72);
    { uint64_t t29 = a16; a16 = o_add(t29, a26); a26 = o_sub(t29, a26); }
    { uint64_t t30 = a21; a21 = o_add(t30, a31); a31 = o_sub(t30, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t31 = a16; a16 = o_add(t31, a21); a21 = o_sub(t31, a21); }
    { uint64_t t32 = a26; a26 = o_add(t32, a31); a31 = o_sub(t32, a31); }
    { uint64_t t33 = a36; a36 = o_add(t33, a6); a6 = o_sub(t33, a6); }
    { uint64_t t34 = a1; a1 = o_add(t34, a11); a11 = o_sub(t34, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t35 = a36; a36 = o_add(t35, a1); a1 = o_sub(t35, a1); }
    { uint64_t t36 = a6; a6 = o_add(t36, a11); a11 = o_sub(t36, a11); }
    { uint64_t t37 = a24; a24 = o_add(t37, a4); a4 = o_sub(t37, a4); }
    { uint64_t t38 = a29; a29 = o_add(t38, a9); a9 = o_sub(t38, a9); }
    { uint64_t t39 = a34; a34 = o_add(t39, a14); a14 = o_sub(t39, a14); }
    { uint64_t t40 = a39; a39 = o_add(t40, a19); a19 = o_sub(t40, a19); }
    a9 = o_shift(a9, 24);
    a14 = o_shift(a14, 48);
    a19 = o_shift(a19, 72);
    { uint64_t t41 = a24; a24 = o_add(t41, a34); a34 = o_sub(t41, a34); }
    { uint64_t t42 = a29; a29 = o_add(t42, a39); a39 = o_sub(t42, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t43 = a24; a24 = o_add(t43, a29); a29 = o_sub(t43, a29); }
    { uint64_t t44 = a34; a34 = o_add(t44, a39); a39 = o_sub(t44, a39); }
    { uint64_t t45 = a4; a4 = o_add(t45, a14); a14 = o_sub(t45, a14); }
    { uint64_t t46 = a9; a9 = o_add(t46, a19); a19 = o_sub(t46, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t47 = a4; a4 = o_add(t47, a9); a9 = o_sub(t47, a9); }
    { uint64_t t48 = a14; a14 = o_add(t48, a19); a19 = o_sub(t48, a19); }
    { uint64_t t49 = a32; a32 = o_add(t49, a12); a12 = o_sub(t49, a12); }
    { uint64_t t50 = a37; a37 = o_add(t50, a17); a17 = o_sub(t50, a17); }
    { uint64_t t51 = a2; a2 = o_add(t51, a22); a22 = o_sub(t51, a22); }
    { uint64_t t52 = a7; a7 = o_add(t52, a27); a27 = o_sub(t52, a27); }
    a17 = o_shift(a17, 24);
    a22 = o_shift(a22, 48);
    a27 = o_shift(a27, 72);
    { uint64_t t53 = a32; a32 = o_add(t53, a2); a2 = o_sub(t53, a2); }
    { uint64_t t54 = a37; a37 = o_add(t54, a7); a7 = o_sub(t54, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t55 = a32; a32 = o_add(t55, a37); a37 = o_sub(t55, a37); }
    { uint64_t t56 = a2; a2 = o_add(t56, a7); a7 = o_sub(t56, a7); }
    { uint64_t t57 = a12; a12 = o_add(t57, a22); a22 = o_sub(t57, a22); }
    { uint64_t t58 = a17; a17 = o_add(t58, a27); a27 = o_sub(t58, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t59 = a12; a12 = o_add(t59, a17); a17 = o_sub(t59, a17); }
    { uint64_t t60 = a22; a22 = o_add(t60, a27); a27 = o_sub(t60, a27); }
    { uint64_t t61 = a8; a8 = o_add(t61, a32); a32 = o_sub(t61, a32); }
    { uint64_t t62 = a24; a24 = o_add(t62, a16); a16 = o_sub(t62, a16); }
    a16 = o_shift(a16, 48);
    { uint64_t t63 = a8; a8 = o_add(t63, a24); a24 = o_sub(t63, a24); }
    { uint64_t t64 = a32; a32 = o_add(t64, a16); a16 = o_sub(t64, a16); }
    uint64_t t65 = a0;
    a0 = o_add(a0, a8);
    a8 = o_mul(a8, 4611686017353646080ULL);
    a32 = o_mul(a32, 16181989089180173841ULL);
    a24 = o_mul(a24, 5818851782451133869ULL);
    a16 = o_mul(a16, 11322249509082494407ULL);
    a8 = o_add(a8, t65);
    { uint64_t t66 = a8; a8 = o_add(t66, a24); a24 = o_sub(t66, a24); }
    { uint64_t t67 = a16; a16 = o_add(t67, a32); a32 = o_sub(t67, a32); }
    a32 = o_shift(a32, 48);
    { uint64_t t68 = a8; a8 = o_add(t68, a16); a16 = o_sub(t68, a16); }
    { uint64_t t69 = a24; a24 = o_add(t69, a32); a32 = o_sub(t69, a32); }
    { uint64_t t70 = a28; a28 = o_add(t70, a12); a12 = o_sub(t70, a12); }
    { uint64_t t71 = a4; a4 = o_add(t71, a36); a36 = o_sub(t71, a36); }
    a36 = o_shift(a36, 48);
    { uint64_t t72 = a28; a28 = o_add(t72, a4); a4 = o_sub(t72, a4); }
    { uint64_t t73 = a12; a12 = o_add(t73, a36); a36 = o_sub(t73, a36); }
    uint64_t t74 = a20;
    a20 = o_add(a20, a28);
    a28 = o_mul(a28, 4611686017353646080ULL);
    a12 = o_mul(a12, 16181989089180173841ULL);
    a4 = o_mul(a4, 5818851782451133869ULL);
    a36 = o_mul(a36, 11322249509082494407ULL);
    a28 = o_add(a28, t74);
    { uint64_t t75 = a28; a28 = o_add(t75, a4); a4 = o_sub(t75, a4); }
    { uint64_t t76 = a36; a36 = o_add(t76, a12); a12 = o_sub(t76, a12); }
    a12 = o_shift(a12, 48);
    { uint64_t t77 = a28; a28 = o_add(t77, a36); a36 = o_sub(t77, a36); }
    { uint64_t t78 = a4; a4 = o_add(t78, a12); a12 = o_sub(t78, a12); }
    { uint64_t t79 = a18; a18 = o_add(t79, a2); a2 = o_sub(t79, a2); }
    { uint64_t t80 = a34; a34 = o_add(t80, a26); a26 = o_sub(t80, a26); }
    a26 = o_shift(a26, 48);
    { uint64_t t81 = a18; a18 = o_add(t81, a34); a34 = o_sub(t81, a34); }
    { uint64_t t82 = a2; a2 = o_add(t82, a26); a26 = o_sub(t82, a26); }
    uint64_t t83 = a10;
    a10 = o_add(a10, a18);
    a18 = o_mul(a18, 4611686017353646080ULL);
    a2 = o_mul(a2, 16181989089180173841ULL);
    a34 = o_mul(a34, 5818851782451133869ULL);
    a26 = o_mul(a26, 11322249509082494407ULL);
    a18 = o_add(a18, t83);
    { uint64_t t84 = a18; a18 = o_add(t84, a34); a34 = o_sub(t84, a34); }
    { uint64_t t85 = a26; a26 = o_add(t85, a2); a2 = o_sub(t85, a2); }
    a2 = o_shift(a2, 48);
    { uint64_t t86 = a18; a18 = o_add(t86, a26); a26 = o_sub(t86, a26); }
    { uint64_t t87 = a34; a34 = o_add(t87, a2); a2 = o_sub(t87, a2); }
    { uint64_t t88 = a38; a38 = o_add(t88, a22); a22 = o_sub(t88, a22); }
    { uint64_t t89 = a14; a14 = o_add(t89, a6); a6 = o_sub(t89, a6); }
    a6 = o_shift(a6, 48);
    { uint64_t t90 = a38; a38 = o_add(t90, a14); a14 = o_sub(t90, a14); }
    { uint64_t t91 = a22; a22 = o_add(t91, a6); a6 = o_sub(t91, a6); }
    uint64_t t92 = a30;
    a30 = o_add(a30, a38);
    a38 = o_mul(a38, 4611686017353646080ULL);
    a22 = o_mul(a22, 16181989089180173841ULL);
    a14 = o_mul(a14, 5818851782451133869ULL);
    a6 = o_mul(a6, 11322249509082494407ULL);
    a38 = o_add(a38, t92);
    { uint64_t t93 = a38; a38 = o_add(t93, a14); a14 = o_sub(t93, a14); }
    { uint64_t t94 = a6; a6 = o_add(t94, a22); a22 = o_sub(t94, a22); }
    a22 = o_shift(a22, 48);
    { uint64_t t95 = a38; a38 = o_add(t95, a6); a6 = o_sub(t95, a6); }
    { uint64_t t96 = a14; a14 = o_add(t96, a22); a22 = o_sub(t96, a22); }
    { uint64_t t97 = a13; a13 = o_add(t97, a37); a37 = o_sub(t97, a37); }
    { uint64_t t98 = a29; a29 = o_add(t98, a21); a21 = o_sub(t98, a21); }
    a21 = o_shift(a21, 48);
    { uint64_t t99 = a13; a13 = o_add(t99, a29); a29 = o_sub(t99, a29); }
    { uint64_t t100 = a37; a37 = o_add(t100, a21); a21 = o_sub(t100, a21); }
    uint64_t t101 = a5;
    a5 = o_add(a5, a13);
    a13 = o_mul(a13, 4611686017353646080ULL);
    a37 = o_mul(a37, 16181989089180173841ULL);
    a29 = o_mul(a29, 5818851782451133869ULL);
    a21 = o_mul(a21, 11322249509082494407ULL);
    a13 = o_add(a13, t101);
    { uint64_t t102 = a13; a13 = o_add(t102, a29); a29 = o_sub(t102, a29); }
    { uint64_t t103 = a21; a21 = o_add(t103, a37); a37 = o_sub(t103, a37); }
    a37 = o_shift(a37, 48);
    { uint64_t t104 = a13; a13 = o_add(t104, a21); a21 = o_sub(t104, a21); }
    { uint64_t t105 = a29; a29 = o_add(t105, a37); a37 = o_sub(t105, a37); }
    { uint64_t t106 = a33; a33 = o_add(t106, a17); a17 = o_sub(t106, a17); }
    { uint64_t t107 = a9; a9 = o_add(t107, a1); a1 = o_sub(t107, a1); }
    a1 = o_shift(a1, 48);
    { uint64_t t108 = a33; a33 = o_add(t108, a9); a9 = o_sub(t108, a9); }
    { uint64_t t109 = a17; a17 = o_add(t109, a1); a1 = o_sub(t109, a1); }
    uint64_t t110 = a25;
    a25 = o_add(a25, a33);
    a33 = o_mul(a33, 4611686017353646080ULL);
    a17 = o_mul(a17, 16181989089180173841ULL);
    a9 = o_mul(a9, 5818851782451133869ULL);
    a1 = o_mul(a1, 11322249509082494407ULL);
    a33 = o_add(a33, t110);
    { uint64_t t111 = a33; a33 = o_add(t111, a9); a9 = o_sub(t111, a9); }
    { uint64_t t112 = a1; a1 = o_add(t112, a17); a17 = o_sub(t112, a17); }
    a17 = o_shift(a17, 48);
    { uint64_t t113 = a33; a33 = o_add(t113, a1); a1 = o_sub(t113, a1); }
    { uint64_t t114 = a9; a9 = o_add(t114, a17); a17 = o_sub(t114, a17); }
    { uint64_t t115 = a23; a23 = o_add(t115, a7); a7 = o_sub(t115, a7); }
    { uint64_t t116 = a39; a39 = o_add(t116, a31); a31 = o_sub(t116, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t117 = a23; a23 = o_add(t117, a39); a39 = o_sub(t117, a39); }
    { uint64_t t118 = a7; a7 = o_add(t118, a31); a31 = o_sub(t118, a31); }
    uint64_t t119 = a15;
    a15 = o_add(a15, a23);
    a23 = o_mul(a23, 4611686017353646080ULL);
    a7 = o_mul(a7, 16181989089180173841ULL);
    a39 = o_mul(a39, 5818851782451133869ULL);
    a31 = o_mul(a31, 11322249509082494407ULL);
    a23 = o_add(a23, t119);
    { uint64_t t120 = a23; a23 = o_add(t120, a39); a39 = o_sub(t120, a39); }
    { uint64_t t121 = a31; a31 = o_add(t121, a7); a7 = o_sub(t121, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t122 = a23; a23 = o_add(t122, a31); a31 = o_sub(t122, a31); }
    { uint64_t t123 = a39; a39 = o_add(t123, a7); a7 = o_sub(t123, a7); }
    { uint64_t t124 = a3; a3 = o_add(t124, a27); a27 = o_sub(t124, a27); }
    { uint64_t t125 = a19; a19 = o_add(t125, a11); a11 = o_sub(t125, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t126 = a3; a3 = o_add(t126, a19); a19 = o_sub(t126, a19); }
    { uint64_t t127 = a27; a27 = o_add(t127, a11); a11 = o_sub(t127, a11); }
    uint64_t t128 = a35;
    a35 = o_add(a35, a3);
    a3 = o_mul(a3, 4611686017353646080ULL);
    a27 = o_mul(a27, 16181989089180173841ULL);
    a19 = o_mul(a19, 5818851782451133869ULL);
    a11 = o_mul(a11, 11322249509082494407ULL);
    a3 = o_add(a3, t128);
    { uint64_t t129 = a3; a3 = o_add(t129, a19); a19 = o_sub(t129, a19); }
    { uint64_t t130 = a11; a11 = o_add(t130, a27); a27 = o_sub(t130, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t131 = a3; a3 = o_add(t131, a11); a11 = o_sub(t131, a11); }
    { uint64_t t132 = a19; a19 = o_add(t132, a27); a27 = o_sub(t132, a27); }
    v[0] = a0;
    v[1] = a28;
    v[2] = a34;
    v[3] = a22;
    v[4] = a21;
    v[5] = a25;
    v[6] = a23;
    v[7] = a19;
    v[8] = a32;
    v[9] = a36;
    v[10] = a10;
    v[11] = a38;
    v[12] = a29;
    v[13] = a17;
    v[14] = a31;
    v[15] = a35;
    v[16] = a8;
    v[17] = a4;
    v[18] = a2;
    v[19] = a6;
    v[20] = a5;
    v[21] = a33;
    v[22] = a39;
    v[23] = a27;
    v[24] = a16;
    v[25] = a20;
    v[26] = a18;
    v[27] = a14;
    v[28] = a37;
    v[29] = a1;
    v[30] = a15;
    v[31] = a3;
    v[32] = a24;
    v[33] = a12;
    v[34] = a26;
    v[35] = a30;
    v[36] = a13;
    v[37] = a9;
    v[38] = a7;
    v[39] = a11;
}

static void o_ntt_48(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33], a34 = v[34], a35 = v[35], a36 = v[36], a37 = v[37], a38 = v[38], a39 = v[39], a40 = v[40], a41 = v[41], a42 = v[42], a43 = v[43], a44 = v[44], a45 = v[45], a46 = v[46], a47 = v[47];
    { uint64_t t1 = a0, t2 = a16, t3 = a32;
      a0 = o_add(o_add(t1, t2), t3);
      a16 = o_sub(o_add(t1, o_shift(t2, 64)), o_shift(t3, 32));
      a32 = o_add(o_sub(t1, o_shift(t2, 32)), o_shift(t3, 64)); }
    { uint64_t t4 = a24, t5 = a40, t6 = a8;
      a24 = o_add(o_add(t4, t5), t6);
      a40 = o_sub(o_add(t4, o_shift(t5, 64)), o_shift(t6, 32));
      a8 = o_add(o_sub(t4, o_shift(t5, 32)), o_shift(t6, 64)); }
    { uint64_t t7 = a0; a0 = o_add(t7, a24); a24 = o_sub(t7, a24); }
    { uint64_t t8 = a16; a16 = o_add(t8, a40); a40 = o_sub(t8, a40); }
    { uint64_t t9 = a32; a32 = o_add(t9, a8); a8 = o_sub(t9, a8); }
    { uint64_t t10 = a1, t11 = a17, t12 = a33;
      a1 = o_add(o_add(t10, t11), t12);
      a17 = o_sub(o_add(t10, o_shift(t11, 64)), o_shift(t12, 32));
      a33 = o_add(o_sub(t10, o_shift(t11, 32)), o_shift(t12, 64)); }
    { uint64_t t13 = a25, t14 = a41, t15 = a9;
      a25 = o_add(o_add(t13, t14), t15);
      a41 = o_sub(o_add(t13, o_shift(t14, 64)), o_shift(t15, 32));
      a9 = o_add(o_sub(t13, o_shift(t14, 32)), o_shift(t15, 64)); }
    { uint64_t t16 = a1; a1 = o_add(t16, a25); a25 = o_sub(t16, a25); }
    { uint64_t t17 = a17; a17 = o_add(t17, a41); a41 = o_sub(t17, a41); }
    { uint64_t t18 = a33; a33 = o_add(t18, a9); a9 = o_sub(t18, a9); }
    { uint64_t t19 = a2, t20 = a18, t21 = a34;
      a2 = o_add(o_add(t19, t20), t21);
      a18 = o_sub(o_add(t19, o_shift(t20, 64)), o_shift(t21, 32));
      a34 = o_add(o_sub(t19, o_shift(t20, 32)), o_shift(t21, 64)); }
    { uint64_t t22 = a26, t23 = a42, t24 = a10;
      a26 = o_add(o_add(t22, t23), t24);
      a42 = o_sub(o_add(t22, o_shift(t23, 64)), o_shift(t24, 32));
      a10 = o_add(o_sub(t22, o_shift(t23, 32)), o_shift(t24, 64)); }
    { uint64_t t25 = a2; a2 = o_add(t25, a26); a26 = o_sub(t25, a26); }
    { uint64_t t26 = a18; a18 = o_add(t26, a42); a42 = o_sub(t26, a42); }
    { uint64_t t27 = a34; a34 = o_add(t27, a10); a10 = o_sub(t27, a10); }
    { uint64_t t28 = a3, t29 = a19, t30 = a35;
      a3 = o_add(o_add(t28, t29), t30);
      a19 = o_sub(o_add(t28, o_shift(t29, 64)), o_shift(t30, 32));
      a35 = o_add(o_sub(t28, o_shift(t29, 32)), o_shift(t30, 64)); }
    { uint64_t t31 = a27, t32 = a43, t33 = a11;
      a27 = o_add(o_add(t31, t32), t33);
      a43 = o_sub(o_add(t31, o_shift(t32, 64)), o_shift(t33, 32));
      a11 = o_add(o_sub(t31, o_shift(t32, 32)), o_shift(t33, 64)); }
    { uint64_t t34 = a3; a3 = o_add(t34, a27); a27 = o_sub(t34, a27); }
    { uint64_t t35 = a19; a19 = o_add(t35, a43); a43 = o_sub(t35, a43); }
    { uint64_t t36 = a35; a35 = o_add(t36, a11); a11 = o_sub(t36, a11); }
    { uint64_t t37 = a4, t38 = a20, t39 = a36;
      a4 = o_add(o_add(t37, t38), t39);
      a20 = o_sub(o_add(t37, o_shift(t38, 64)), o_shift(t39, 32));
      a36 = o_add(o_sub(t37, o_shift(t38, 32)), o_shift(t39, 64)); }
    { uint64_t t40 = a28, t41 = a44, t42 = a12;
      a28 = o_add(o_add(t40, t41), t42);
      a44 = o_sub(o_add(t40, o_shift(t41, 64)), o_shift(t42, 32));
      a12 = o_add(o_sub(t40, o_shift(t41, 32)), o_shift(t42, 64)); }
    { uint64_t t43 = a4; a4 = o_add(t43, a28); a28 = o_sub(t43, a28); }
    { uint64_t t44 = a20; a20 = o_add(t44, a44); a44 = o_sub(t44, a44); }
    { uint64_t t45 = a36; a36 = o_add(t45, a12); a12 = o_sub(t45, a12); }
    { uint64_t t46 = a5, t47 = a21, t48 = a37;
      a5 = o_add(o_add(t46, t47), t48);
      a21 = o_sub(o_add(t46, o_shift(t47, 64)), o_shift(t48, 32));
      a37 = o_add(o_sub(t46, o_shift(t47, 32)), o_shift(t48, 64)); }
    { uint64_t t49 = a29, t50 = a45, t51 = a13;
      a29 = o_add(o_add(t49, t50), t51);
      a45 = o_sub(o_add(t49, o_shift(t50, 64)), o_shift(t51, 32));
      a13 = o_add(o_sub(t49, o_shift(t50, 32)), o_shift(t51, 64)); }
    { uint64_t t52 = a5; a5 = o_add(t52, a29); a29 = o_sub(t52, a29); }
    { uint64_t t53 = a21; a21 = o_add(t53, a45); a45 = o_sub(t53, a45); }
    { uint64_t t54 = a37; a37 = o_add(t54, a13); a13 = o_sub(t54, a13); }
    { uint64_t t55 = a6, t56 = a22, t57 = a38;
      a6 = o_add(o_add(t55, t56), t57);
      a22 = o_sub(o_add(t55, o_shift(t56, 64)), o_shift(t57, 32));
      a38 = o_add(o_sub(t55, o_shift(t56, 32)), o_shift(t57, 64)); }
    { uint64_t t58 = a30, t59 = a46, t60 = a14;
      a30 = o_add(o_add(t58, t59), t60);
      a46 = o_sub(o_add(t58, o_shift(t59, 64)), o_shift(t60, 32));
      a14 = o_add(o_sub(t58, o_shift(t59, 32)), o_shift(t60, 64)); }
    { uint64_t t61 = a6; a6 = o_add(t61, a30); a30 = o_sub(t61, a30); }
    { uint64_t t62 = a22; a22 = o_add(t62, a46); a46 = o_sub(t62, a46); }
    { uint64_t t63 = a38; a38 = o_add(t63, a14); a14 = o_sub(t63, a14); }
    { uint64_t t64 = a7, t65 = a23, t66 = a39;
      a7 = o_add(o_add(t64, t65), t66);
      a23 = o_sub(o_add(t64, o_shift(t65, 64)), o_shift(t66, 32));
      a39 = o_add(o_sub(t64, o_shift(t65, 32)), o_shift(t66, 64)); }
    { uint64_t t67 = a31, t68 = a47, t69 = a15;
      a31 = o_add(o_add(t67, t68), t69);
      a47 = o_sub(o_add(t67, o_shift(t68, 64)), o_shift(t69, 32));
      a15 = o_add(o_sub(t67, o_shift(t68, 32)), o_shift(t69, 64)); }
    { uint64_t t70 = a7; a7 = o_add(t70, a31); a31 = o_sub(t70, a31); }
    { uint64_t t71 = a23; a23 = o_add(t71, a47); a47 = o_sub(t71, a47); }
    { uint64_t t72 = a39; a39 = o_add(t72, a15); a15 = o_sub(t72, a15); }
    a41 = o_shift(a41, 4);
    a33 = o_shift(a33, 8);
    a25 = o_shift(a25, 12);
    a17 = o_shift(a17, 16);
    a9 = o_shift(a9, 20);
    a42 = o_shift(a42, 8);
    a34 = o_shift(a34, 16);
    a26 = o_shift(a26, 24);
    a18 = o_shift(a18, 32);
    a10 = o_shift(a10, 40);
    a43 = o_shift(a43, 12);
    a35 = o_shift(a35, 24);
    a27 = o_shift(a27, 36);
    a19 = o_shift(a19, 48);
    a11 = o_shift(a11, 60);
    a44 = o_shift(a44, 16);
    a36 = o_shift(a36, 32);
    a28 = o_shift(a28, 48);
    a20 = o_shift(a20, 64);
    a12 = o_shift(a12, 80);
    a45 = o_shift(a45, 20);
    a37 = o_shift(a37, 40);
    a29 = o_shift(a29, 60);
    a21 = o_shift(a21, 80);
    a13 = o_neg(o_shift(a13, 4));
    a46 = o_shift(a46, 24);
    a38 = o_shift(a38, 48);
    a30 = o_shift(a30, 72);
    a22 = o_neg(a22);
    a14 = o_neg(o_shift(a14, 24));
    a47 = o_shift(a47, 28);
    a39 = o_shift(a39, 56);
    a31 = o_shift(a31, 84);
    a23 = o_neg(o_shift(a23, 16));
    a15 = o_neg(o_shift(a15, 44));
    { uint64_t t73 = a0; a0 = o_add(t73, a4); a4 = o_sub(t73, a4); }
    { uint64_t t74 = a1; a1 = o_add(t74, a5); a5 = o_sub(t74, a5); }
    { uint64_t t75 = a2; a2 = o_add(t75, a6); a6 = o_sub(t75, a6); }
    { uint64_t t76 = a3; a3 = o_add(t76, a7); a7 = o_sub(t76, a7); }
    a5 = o_shift(a5, 24);
    a6 = o_shift(a6, 48);
    a7 = o_shift(a7, 72);
    { uint64_t t77 = a0; a0 = o_add(t77, a2); a2 = o_sub(t77, a2); }
    { uint64_t t78 = a1; a1 = o_add(t78, a3); a3 = o_sub(t78, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t79 = a0; a0 = o_add(t79, a1); a1 = o_sub(t79, a1); }
    { uint64_t t80 = a2; a2 = o_add(t80, a3); a3 = o_sub(t80, a3); }
    { uint64_t t81 = a4; a4 = o_add(t81, a6); a6 = o_sub(t81, a6); }
    { uint64_t t82 = a5; a5 = o_add(t82, a7); a7 = o_sub(t82, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t83 = a4; a4 = o_add(t83, a5); a5 = o_sub(t83, a5); }
    { uint64_t t84 = a6; a6 = o_add(t84, a7); a7 = o_sub(t84, a7); }
    { uint64_t t85 = a40; a40 = o_add(t85, a44); a44 = o_sub(t85, a44); }
    { uint64_t t86 = a41; a41 = o_add(t86, a45); a45 = o_sub(t86, a45); }
    { uint64_t t87 = a42; a42 = o_add(t87, a46); a46 = o_sub(t87, a46); }
    { uint64_t t88 = a43; a43 = o_add(t88, a47); a47 = o_sub(t88, a47); }
    a45 = o_shift(a45, 24);
    a46 = o_shift(a46, 48);
    a47 = o_shift(a47, 72);
    { uint64_t t89 = a40; a40 = o_add(t89, a42); a42 = o_sub(t89, a42); }
    { uint64_t t90 = a41; a41 = o_add(t90, a43); a43 = o_sub(t90, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t91 = a40; a40 = o_add(t91, a41); a41 = o_sub(t91, a41); }
    { uint64_t t92 = a42; a42 = o_add(t92, a43); a43 = o_sub(t92, a43); }
    { uint64_t t93 = a44; a44 = o_add(t93, a46); a46 = o_sub(t93, a46); }
    { uint64_t t94 = a45; a45 = o_add(t94, a47); a47 = o_sub(t94, a47); }
    a47 = o_shift(a47, 48);
    { uint64_t t95 = a44; a44 = o_add(t95, a45); a45 = o_sub(t95, a45); }
    { uint64_t t96 = a46; a46 = o_add(t96, a47); a47 = o_sub(t96, a47); }
    { uint64_t t97 = a32; a32 = o_add(t97, a36); a36 = o_sub(t97, a36); }
    { uint64_t t98 = a33; a33 = o_add(t98, a37); a37 = o_sub(t98, a37); }
    { uint64_t t99 = a34; a34 = o_add(t99, a38); a38 = o_sub(t99, a38); }
    { uint64_t t100 = a35; a35 = o_add(t100, a39); a39 = o_sub(t100, a39); }
    a37 = o_shift(a37, 24);
    a38 = o_shift(a38, 48);
    a39 = o_shift(a39, 72);
    { uint64_t t101 = a32; a32 = o_add(t101, a34); a34 = o_sub(t101, a34); }
    { uint64_t t102 = a33; a33 = o_add(t102, a35); a35 = o_sub(t102, a35); }
    a35 = o_shift(a35, 48);
    { uint64_t t103 = a32; a32 = o_add(t103, a33); a33 = o_sub(t103, a33); }
    { uint64_t t104 = a34; a34 = o_add(t104, a35); a35 = o_sub(t104, a35); }
    { uint64_t t105 = a36; a36 = o_add(t105, a38); a38 = o_sub(t105, a38); }
    { uint64_t t106 = a37; a37 = o_add(t106, a39); a39 = o_sub(t106, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t107 = a36; a36 = o_add(t107, a37); a37 = o_sub(t107, a37); }
    { uint64_t t108 = a38; a38 = o_add(t108, a39); a39 = o_sub(t108, a39); }
    { uint64_t t109 = a24; a24 = o_add(t109, a28); a28 = o_sub(t109, a28); }
    { uint64_t t110 = a25; a25 = o_add(t110, a29); a29 = o_sub(t110, a29); }
    { uint64_t t111 = a26; a26 = o_add(t111, a30); a30 = o_sub(t111, a30); }
    { uint64_t t112 = a27; a27 = o_add(t112, a31); a31 = o_sub(t112, a31); }
    a29 = o_shift(a29, 24);
    a30 = o_shift(a30, 48);
    a31 = o_shift(a31, 72);
    { uint64_t t113 = a24; a24 = o_add(t113, a26); a26 = o_sub(t113, a26); }
    { uint64_t t114 = a25; a25 = o_add(t114, a27); a27 = o_sub(t114, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t115 = a24; a24 = o_add(t115, a25); a25 = o_sub(t115, a25); }
    { uint64_t t116 = a26; a26 = o_add(t116, a27); a27 = o_sub(t116, a27); }
    { uint64_t t117 = a28; a28 = o_add(t117, a30); a30 = o_sub(t117, a30); }
    { uint64_t t118 = a29; a29 = o_add(t118, a31); a31 = o_sub(t118, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t119 = a28; a28 = o_add(t119, a29); a29 = o_sub(t119, a29); }
    { uint64_t t120 = a30; a30 = o_add(t120, a31); a31 = o_sub(t120, a31); }
    { uint64_t t121 = a16; a16 = o_add(t121, a20); a20 = o_sub(t121, a20); }
    { uint64_t t122 = a17; a17 = o_add(t122, a21); a21 = o_sub(t122, a21); }
    { uint64_t t123 = a18; a18 = o_add(t123, a22); a22 = o_sub(t123, a22); }
    { uint64_t t124 = a19; a19 = o_add(t124, a23); a23 = o_sub(t124, a23); }
    a21 = o_shift(a21, 24);
    a22 = o_shift(a22, 48);
    a23 = o_shift(a23, 72);
    { uint64_t t125 = a16; a16 = o_add(t125, a18); a18 = o_sub(t125, a18); }
    { uint64_t t126 = a17; a17 = o_add(t126, a19); a19 = o_sub(t126, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t127 = a16; a16 = o_add(t127, a17); a17 = o_sub(t127, a17); }
    { uint64_t t128 = a18; a18 = o_add(t128, a19); a19 = o_sub(t128, a19); }
    { uint64_t t129 = a20; a20 = o_add(t129, a22); a22 = o_sub(t129, a22); }
    { uint64_t t130 = a21; a21 = o_add(t130, a23); a23 = o_sub(t130, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t131 = a20; a20 = o_add(t131, a21); a21 = o_sub(t131, a21); }
    { uint64_t t132 = a22; a22 = o_add(t132, a23); a23 = o_sub(t132, a23); }
    { uint64_t t133 = a8; a8 = o_add(t133, a12); a12 = o_sub(t133, a12); }
    { uint64_t t134 = a9; a9 = o_add(t134, a13); a13 = o_sub(t134, a13); }
    { uint64_t t135 = a10; a10 = o_add(t135, a14); a14 = o_sub(t135, a14); }
    { uint64_t t136 = a11; a11 = o_add(t136, a15); a15 = o_sub(t136, a15); }
    a13 = o_shift(a13, 24);
    a14 = o_shift(a14, 48);
    a15 = o_shift(a15, 72);
    { uint64_t t137 = a8; a8 = o_add(t137, a10); a10 = o_sub(t137, a10); }
    { uint64_t t138 = a9; a9 = o_add(t138, a11); a11 = o_sub(t138, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t139 = a8; a8 = o_add(t139, a9); a9 = o_sub(t139, a9); }
    { uint64_t t140 = a10; a10 = o_add(t140, a11); a11 = o_sub(t140, a11); }
    { uint64_t t141 = a12; a12 = o_add(t141, a14); a14 = o_sub(t141, a14); }
    { uint64_t t142 = a13; a13 = o_add(t142, a15); a15 = o_sub(t142, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t143 = a12; a12 = o_add(t143, a13); a13 = o_sub(t143, a13); }
    { uint64_t t144 = a14; a14 = o_add(t144, a15); a15 = o_sub(t144, a15); }
    v[0] = a0;
    v[1] = a40;
    v[2] = a32;
    v[3] = a24;
    v[4] = a16;
    v[5] = a8;
    v[6] = a4;
    v[7] = a44;
    v[8] = a36;
    v[9] = a28;
    v[10] = a20;
    v[11] = a12;
    v[12] = a2;
    v[13] = a42;
    v[14] = a34;
    v[15] = a26;
    v[16] = a18;
    v[17] = a10;
    v[18] = a6;
    v[19] = a46;
    v[20] = a38;
    v[21] = a30;
    v[22] = a22;
    v[23] = a14;
    v[24] = a1;
    v[25] = a41;
    v[26] = a33;
    v[27] = a25;
    v[28] = a17;
    v[29] = a9;
    v[30] = a5;
    v[31] = a45;
    v[32] = a37;
    v[33] = a29;
    v[34] = a21;
    v[35] = a13;
    v[36] = a3;
    v[37] = a43;
    v[38] = a35;
    v[39] = a27;
    v[40] = a19;
    v[41] = a11;
    v[42] = a7;
    v[43] = a47;
    v[44] = a39;
    v[45] = a31;
    v[46] = a23;
    v[47] = a15;
}

static void o_ntt_51(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33], a34 = v[34], a35 = v[35], a36 = v[36], a37 = v[37], a38 = v[38], a39 = v[39], a40 = v[40], a41 = v[41], a42 = v[42], a43 = v[43], a44 = v[44], a45 = v[45], a46 = v[46], a47 = v[47], a48 = v[48], a49 = v[49], a50 = v[50];
    { uint64_t t1 = a3; a3 = o_add(t1, a48); a48 = o_sub(t1, a48); }
    { uint64_t t2 = a12; a12 = o_add(t2, a39); a39 = o_sub(t2, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t3 = a3; a3 = o_add(t3, a12); a12 = o_sub(t3, a12); }
    { uint64_t t4 = a48; a48 = o_add(t4, a39); a39 = o_sub(t4, a39); }
    { uint64_t t5 = a18; a18 = o_add(t5, a33); a33 = o_sub(t5, a33); }
    { uint64_t t6 = a21; a21 = o_add(t6, a30); a30 = o_sub(t6, a30); }
    a30 = o_shift(a30, 48);
    { uint64_t t7 = a18; a18 = o_add(t7, a21); a21 = o_sub(t7, a21); }
    { uint64_t t8 = a33; a33 = o_add(t8, a30); a30 = o_sub(t8, a30); }
    { uint64_t t9 = a6; a6 = o_add(t9, a45); a45 = o_sub(t9, a45); }
    { uint64_t t10 = a24; a24 = o_add(t10, a27); a27 = o_sub(t10, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t11 = a6; a6 = o_add(t11, a24); a24 = o_sub(t11, a24); }
    { uint64_t t12 = a45; a45 = o_add(t12, a27); a27 = o_sub(t12, a27); }
    { uint64_t t13 = a36; a36 = o_add(t13, a15); a15 = o_sub(t13, a15); }
    { uint64_t t14 = a42; a42 = o_add(t14, a9); a9 = o_sub(t14, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t15 = a36; a36 = o_add(t15, a42); a42 = o_sub(t15, a42); }
    { uint64_t t16 = a15; a15 = o_add(t16, a9); a9 = o_sub(t16, a9); }
    a33 = o_shift(a33, 12);
    a21 = o_shift(a21, 24);
    a30 = o_shift(a30, 36);
    a45 = o_shift(a45, 24);
    a24 = o_shift(a24, 48);
    a27 = o_shift(a27, 72);
    a15 = o_shift(a15, 36);
    a42 = o_shift(a42, 72);
    a9 = o_neg(o_shift(a9, 12));
    { uint64_t t17 = a3; a3 = o_add(t17, a6); a6 = o_sub(t17, a6); }
    { uint64_t t18 = a18; a18 = o_add(t18, a36); a36 = o_sub(t18, a36); }
    a36 = o_shift(a36, 48);
    { uint64_t t19 = a3; a3 = o_add(t19, a18); a18 = o_sub(t19, a18); }
    { uint64_t t20 = a6; a6 = o_add(t20, a36); a36 = o_sub(t20, a36); }
    { uint64_t t21 = a48; a48 = o_add(t21, a45); a45 = o_sub(t21, a45); }
    { uint64_t t22 = a33; a33 = o_add(t22, a15); a15 = o_sub(t22, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t23 = a48; a48 = o_add(t23, a33); a33 = o_sub(t23, a33); }
    { uint64_t t24 = a45; a45 = o_add(t24, a15); a15 = o_sub(t24, a15); }
    { uint64_t t25 = a12; a12 = o_add(t25, a24); a24 = o_sub(t25, a24); }
    { uint64_t t26 = a21; a21 = o_add(t26, a42); a42 = o_sub(t26, a42); }
    a42 = o_shift(a42, 48);
    { uint64_t t27 = a12; a12 = o_add(t27, a21); a21 = o_sub(t27, a21); }
    { uint64_t t28 = a24; a24 = o_add(t28, a42); a42 = o_sub(t28, a42); }
    { uint64_t t29 = a39; a39 = o_add(t29, a27); a27 = o_sub(t29, a27); }
    { uint64_t t30 = a30; a30 = o_add(t30, a9); a9 = o_sub(t30, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t31 = a39; a39 = o_add(t31, a30); a30 = o_sub(t31, a30); }
    { uint64_t t32 = a27; a27 = o_add(t32, a9); a9 = o_sub(t32, a9); }
    uint64_t t33 = a0;
    a0 = o_add(a0, a3);
    a3 = o_mul(a3, 1152921504338411520ULL);
    a48 = o_mul(a48, 6259776822214049175ULL);
    a12 = o_mul(a12, 9380094172986290191ULL);
    a39 = o_mul(a39, 891943630314919127ULL);
    a6 = o_mul(a6, 17228171707553225791ULL);
    a45 = o_mul(a45, 12855743360534130886ULL);
    a24 = o_mul(a24, 6167687396920564837ULL);
    a27 = o_mul(a27, 17201834061724655524ULL);
    a18 = o_mul(a18, 15308299771656910737ULL);
    a33 = o_mul(a33, 18186005861103657533ULL);
    a21 = o_mul(a21, 53595491891823545ULL);
    a30 = o_mul(a30, 1906638201581172103ULL);
    a36 = o_mul(a36, 18303651001328874822ULL);
    a15 = o_mul(a15, 3077466521755967626ULL);
    a42 = o_mul(a42, 12423593102987598328ULL);
    a9 = o_mul(a9, 18361513053649472048ULL);
    a3 = o_add(a3, t33);
    { uint64_t t34 = a3; a3 = o_add(t34, a18); a18 = o_sub(t34, a18); }
    { uint64_t t35 = a36; a36 = o_add(t35, a6); a6 = o_sub(t35, a6); }
    a6 = o_shift(a6, 48);
    { uint64_t t36 = a3; a3 = o_add(t36, a36); a36 = o_sub(t36, a36); }
    { uint64_t t37 = a18; a18 = o_add(t37, a6); a6 = o_sub(t37, a6); }
    { uint64_t t38 = a9; a9 = o_add(t38, a27); a27 = o_sub(t38, a27); }
    { uint64_t t39 = a30; a30 = o_add(t39, a39); a39 = o_sub(t39, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t40 = a9; a9 = o_add(t40, a30); a30 = o_sub(t40, a30); }
    { uint64_t t41 = a27; a27 = o_add(t41, a39); a39 = o_sub(t41, a39); }
    { uint64_t t42 = a42; a42 = o_add(t42, a24); a24 = o_sub(t42, a24); }
    { uint64_t t43 = a21; a21 = o_add(t43, a12); a12 = o_sub(t43, a12); }
    a12 = o_shift(a12, 48);
    { uint64_t t44 = a42; a42 = o_add(t44, a21); a21 = o_sub(t44, a21); }
    { uint64_t t45 = a24; a24 = o_add(t45, a12); a12 = o_sub(t45, a12); }
    { uint64_t t46 = a15; a15 = o_add(t46, a45); a45 = o_sub(t46, a45); }
    { uint64_t t47 = a33; a33 = o_add(t47, a48); a48 = o_sub(t47, a48); }
    a48 = o_shift(a48, 48);
    { uint64_t t48 = a15; a15 = o_add(t48, a33); a33 = o_sub(t48, a33); }
    { uint64_t t49 = a45; a45 = o_add(t49, a48); a48 = o_sub(t49, a48); }
    a27 = o_shift(a27, 12);
    a30 = o_shift(a30, 24);
    a39 = o_shift(a39, 36);
    a24 = o_shift(a24, 24);
    a21 = o_shift(a21, 48);
    a12 = o_shift(a12, 72);
    a45 = o_shift(a45, 36);
    a33 = o_shift(a33, 72);
    a48 = o_neg(o_shift(a48, 12));
    { uint64_t t50 = a3; a3 = o_add(t50, a42); a42 = o_sub(t50, a42); }
    { uint64_t t51 = a9; a9 = o_add(t51, a15); a15 = o_sub(t51, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t52 = a3; a3 = o_add(t52, a9); a9 = o_sub(t52, a9); }
    { uint64_t t53 = a42; a42 = o_add(t53, a15); a15 = o_sub(t53, a15); }
    { uint64_t t54 = a18; a18 = o_add(t54, a24); a24 = o_sub(t54, a24); }
    { uint64_t t55 = a27; a27 = o_add(t55, a45); a45 = o_sub(t55, a45); }
    a45 = o_shift(a45, 48);
    { uint64_t t56 = a18; a18 = o_add(t56, a27); a27 = o_sub(t56, a27); }
    { uint64_t t57 = a24; a24 = o_add(t57, a45); a45 = o_sub(t57, a45); }
    { uint64_t t58 = a36; a36 = o_add(t58, a21); a21 = o_sub(t58, a21); }
    { uint64_t t59 = a30; a30 = o_add(t59, a33); a33 = o_sub(t59, a33); }
    a33 = o_shift(a33, 48);
    { uint64_t t60 = a36; a36 = o_add(t60, a30); a30 = o_sub(t60, a30); }
    { uint64_t t61 = a21; a21 = o_add(t61, a33); a33 = o_sub(t61, a33); }
    { uint64_t t62 = a6; a6 = o_add(t62, a12); a12 = o_sub(t62, a12); }
    { uint64_t t63 = a39; a39 = o_add(t63, a48); a48 = o_sub(t63, a48); }
    a48 = o_shift(a48, 48);
    { uint64_t t64 = a6; a6 = o_add(t64, a39); a39 = o_sub(t64, a39); }
    { uint64_t t65 = a12; a12 = o_add(t65, a48); a48 = o_sub(t65, a48); }
    { uint64_t t66 = a20; a20 = o_add(t66, a14); a14 = o_sub(t66, a14); }
    { uint64_t t67 = a29; a29 = o_add(t67, a5); a5 = o_sub(t67, a5); }
    a5 = o_shift(a5, 48);
    { uint64_t t68 = a20; a20 = o_add(t68, a29); a29 = o_sub(t68, a29); }
    { uint64_t t69 = a14; a14 = o_add(t69, a5); a5 = o_sub(t69, a5); }
    { uint64_t t70 = a35; a35 = o_add(t70, a50); a50 = o_sub(t70, a50); }
    { uint64_t t71 = a38; a38 = o_add(t71, a47); a47 = o_sub(t71, a47); }
    a47 = o_shift(a47, 48);
    { uint64_t t72 = a35; a35 = o_add(t72, a38); a38 = o_sub(t72, a38); }
    { uint64_t t73 = a50; a50 = o_add(t73, a47); a47 = o_sub(t73, a47); }
    { uint64_t t74 = a23; a23 = o_add(t74, a11); a11 = o_sub(t74, a11); }
    { uint64_t t75 = a41; a41 = o_add(t75, a44); a44 = o_sub(t75, a44); }
    a44 = o_shift(a44, 48);
    { uint64_t t76 = a23; a23 = o_add(t76, a41); a41 = o_sub(t76, a41); }
    { uint64_t t77 = a11; a11 = o_add(t77, a44); a44 = o_sub(t77, a44); }
    { uint64_t t78 = a2; a2 = o_add(t78, a32); a32 = o_sub(t78, a32); }
    { uint64_t t79 = a8; a8 = o_add(t79, a26); a26 = o_sub(t79, a26); }
    a26 = o_shift(a26, 48);
    { uint64_t t80 = a2; a2 = o_add(t80, a8); a8 = o_sub(t80, a8); }
    { uint64_t t81 = a32; a32 = o_add(t81, a26); a26 = o_sub(t81, a26); }
    a50 = o_shift(a50, 12);
    a38 = o_shift(a38, 24);
    a47 = o_shift(a47, 36);
    a11 = o_shift(a11, 24);
    a41 = o_shift(a41, 48);
    a44 = o_shift(a44, 72);
    a32 = o_shift(a32, 36);
    a8 = o_shift(a8, 72);
    a26 = o_neg(o_shift(a26, 12));
    { uint64_t t82 = a20; a20 = o_add(t82, a23); a23 = o_sub(t82, a23); }
    { uint64_t t83 = a35; a35 = o_add(t83, a2); a2 = o_sub(t83, a2); }
    a2 = o_shift(a2, 48);
    { uint64_t t84 = a20; a20 = o_add(t84, a35); a35 = o_sub(t84, a35); }
    { uint64_t t85 = a23; a23 = o_add(t85, a2); a2 = o_sub(t85, a2); }
    { uint64_t t86 = a14; a14 = o_add(t86, a11); a11 = o_sub(t86, a11); }
    { uint64_t t87 = a50; a50 = o_add(t87, a32); a32 = o_sub(t87, a32); }
    a32 = o_shift(a32, 48);
    { uint64_t t88 = a14; a14 = o_add(t88, a50); a50 = o_sub(t88, a50); }
    { uint64_t t89 = a11; a11 = o_add(t89, a32); a32 = o_sub(t89, a32); }
    { uint64_t t90 = a29; a29 = o_add(t90, a41); a41 = o_sub(t90, a41); }
    { uint64_t t91 = a38; a38 = o_add(t91, a8); a8 = o_sub(t91, a8); }
    a8 = o_shift(a8, 48);
    { uint64_t t92 = a29; a29 = o_add(t92, a38); a38 = o_sub(t92, a38); }
    { uint64_t t93 = a41; a41 = o_add(t93, a8); a8 = o_sub(t93, a8); }
    { uint64_t t94 = a5; a5 = o_add(t94, a44); a44 = o_sub(t94, a44); }
    { uint64_t t95 = a47; a47 = o_add(t95, a26); a26 = o_sub(t95, a26); }
    a26 = o_shift(a26, 48);
    { uint64_t t96 = a5; a5 = o_add(t96, a47); a47 = o_sub(t96, a47); }
    { uint64_t t97 = a44; a44 = o_add(t97, a26); a26 = o_sub(t97, a26); }
    uint64_t t98 = a17;
    a17 = o_add(a17, a20);
    a20 = o_mul(a20, 1152921504338411520ULL);
    a14 = o_mul(a14, 6259776822214049175ULL);
    a29 = o_mul(a29, 9380094172986290191ULL);
    a5 = o_mul(a5, 891943630314919127ULL);
    a23 = o_mul(a23, 17228171707553225791ULL);
    a11 = o_mul(a11, 12855743360534130886ULL);
    a41 = o_mul(a41, 6167687396920564837ULL);
    a44 = o_mul(a44, 17201834061724655524ULL);
    a35 = o_mul(a35, 15308299771656910737ULL);
    a50 = o_mul(a50, 18186005861103657533ULL);
    a38 = o_mul(a38, 53595491891823545ULL);
    a47 = o_mul(a47, 1906638201581172103ULL);
    a2 = o_mul(a2, 18303651001328874822ULL);
    a32 = o_mul(a32, 3077466521755967626ULL);
    a8 = o_mul(a8, 12423593102987598328ULL);
    a26 = o_mul(a26, 18361513053649472048ULL);
    a20 = o_add(a20, t98);
    { uint64_t t99 = a20; a20 = o_add(t99, a35); a35 = o_sub(t99, a35); }
    { uint64_t t100 = a2; a2 = o_add(t100, a23); a23 = o_sub(t100, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t101 = a20; a20 = o_add(t101, a2); a2 = o_sub(t101, a2); }
    { uint64_t t102 = a35; a35 = o_add(t102, a23); a23 = o_sub(t102, a23); }
    { uint64_t t103 = a26; a26 = o_add(t103, a44); a44 = o_sub(t103, a44); }
    { uint64_t t104 = a47; a47 = o_add(t104, a5); a5 = o_sub(t104, a5); }
    a5 = o_shift(a5, 48);
    { uint64_t t105 = a26; a26 = o_add(t105, a47); a47 = o_sub(t105, a47); }
    { uint64_t t106 = a44; a44 = o_add(t106, a5); a5 = o_sub(t106, a5); }
    { uint64_t t107 = a8; a8 = o_add(t107, a41); a41 = o_sub(t107, a41); }
    { uint64_t t108 = a38; a38 = o_add(t108, a29); a29 = o_sub(t108, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t109 = a8; a8 = o_add(t109, a38); a38 = o_sub(t109, a38); }
    { uint64_t t110 = a41; a41 = o_add(t110, a29); a29 = o_sub(t110, a29); }
    { uint64_t t111 = a32; a32 = o_add(t111, a11); a11 = o_sub(t111, a11); }
    { uint64_t t112 = a50; a50 = o_add(t112, a14); a14 = o_sub(t112, a14); }
    a14 = o_shift(a14, 48);
    { uint64_t t113 = a32; a32 = o_add(t113, a50); a50 = o_sub(t113, a50); }
    { uint64_t t114 = a11; a11 = o_add(t114, a14); a14 = o_sub(t114, a14); }
    a44 = o_shift(a44, 12);
    a47 = o_shift(a47, 24);
    a5 = o_shift(a5, 36);
    a41 = o_shift(a41, 24);
    a38 = o_shift(a38, 48);
    a29 = o_shift(a29, 72);
    a11 = o_shift(a11, 36);
    a50 = o_shift(a50, 72);
    a14 = o_neg(o_shift(a14, 12));
    { uint64_t t115 = a20; a20 = o_add(t115, a8); a8 = o_sub(t115, a8); }
    { uint64_t t116 = a26; a26 = o_add(t116, a32); a32 = o_sub(t116, a32); }
    a32 = o_shift(a32, 48);
    { uint64_t t117 = a20; a20 = o_add(t117, a26); a26 = o_sub(t117, a26); }
    { uint64_t t118 = a8; a8 = o_add(t118, a32); a32 = o_sub(t118, a32); }
    { uint64_t t119 = a35; a35 = o_add(t119, a41); a41 = o_sub(t119, a41); }
    { uint64_t t120 = a44; a44 = o_add(t120, a11); a11 = o_sub(t120, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t121 = a35; a35 = o_add(t121, a44); a44 = o_sub(t121, a44); }
    { uint64_t t122 = a41; a41 = o_add(t122, a11); a11 = o_sub(t122, a11); }
    { uint64_t t123 = a2; a2 = o_add(t123, a38); a38 = o_sub(t123, a38); }
    { uint64_t t124 = a47; a47 = o_add(t124, a50); a50 = o_sub(t124, a50); }
    a50 = o_shift(a50, 48);
    { uint64_t t125 = a2; a2 = o_add(t125, a47); a47 = o_sub(t125, a47); }
    { uint64_t t126 = a38; a38 = o_add(t126, a50); a50 = o_sub(t126, a50); }
    { uint64_t t127 = a23; a23 = o_add(t127, a29); a29 = o_sub(t127, a29); }
    { uint64_t t128 = a5; a5 = o_add(t128, a14); a14 = o_sub(t128, a14); }
    a14 = o_shift(a14, 48);
    { uint64_t t129 = a23; a23 = o_add(t129, a5); a5 = o_sub(t129, a5); }
    { uint64_t t130 = a29; a29 = o_add(t130, a14); a14 = o_sub(t130, a14); }
    { uint64_t t131 = a37; a37 = o_add(t131, a31); a31 = o_sub(t131, a31); }
    { uint64_t t132 = a46; a46 = o_add(t132, a22); a22 = o_sub(t132, a22); }
    a22 = o_shift(a22, 48);
    { uint64_t t133 = a37; a37 = o_add(t133, a46); a46 = o_sub(t133, a46); }
    { uint64_t t134 = a31; a31 = o_add(t134, a22); a22 = o_sub(t134, a22); }
    { uint64_t t135 = a1; a1 = o_add(t135, a16); a16 = o_sub(t135, a16); }
    { uint64_t t136 = a4; a4 = o_add(t136, a13); a13 = o_sub(t136, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t137 = a1; a1 = o_add(t137, a4); a4 = o_sub(t137, a4); }
    { uint64_t t138 = a16; a16 = o_add(t138, a13); a13 = o_sub(t138, a13); }
    { uint64_t t139 = a40; a40 = o_add(t139, a28); a28 = o_sub(t139, a28); }
    { uint64_t t140 = a7; a7 = o_add(t140, a10); a10 = o_sub(t140, a10); }
    a10 = o_shift(a10, 48);
    { uint64_t t141 = a40; a40 = o_add(t141, a7); a7 = o_sub(t141, a7); }
    { uint64_t t142 = a28; a28 = o_add(t142, a10); a10 = o_sub(t142, a10); }
    { uint64_t t143 = a19; a19 = o_add(t143, a49); a49 = o_sub(t143, a49); }
    { uint64_t t144 = a25; a25 = o_add(t144, a43); a43 = o_sub(t144, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t145 = a19; a19 = o_add(t145, a25); a25 = o_sub(t145, a25); }
    { uint64_t t146 = a49; a49 = o_add(t146, a43); a43 = o_sub(t146, a43); }
    a16 = o_shift(a16, 12);
    a4 = o_shift(a4, 24);
    a13 = o_shift(a13, 36);
    a28 = o_shift(a28, 24);
    a7 = o_shift(a7, 48);
    a10 = o_shift(a10, 72);
    a49 = o_shift(a49, 36);
    a25 = o_shift(a25, 72);
    a43 = o_neg(o_shift(a43, 12));
    { uint64_t t147 = a37; a37 = o_add(t147, a40); a40 = o_sub(t147, a40); }
    { uint64_t t148 = a1; a1 = o_add(t148, a19); a19 = o_sub(t148, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t149 = a37; a37 = o_add(t149, a1); a1 = o_sub(t149, a1); }
    { uint64_t t150 = a40; a40 = o_add(t150, a19); a19 = o_sub(t150, a19); }
    { uint64_t t151 = a31; a31 = o_add(t151, a28); a28 = o_sub(t151, a28); }
    { uint64_t t152 = a16; a16 = o_add(t152, a49); a49 = o_sub(t152, a49); }
    a49 = o_shift(a49, 48);
    { uint64_t t153 = a31; a31 = o_add(t153, a16); a16 = o_sub(t153, a16); }
    { uint64_t t154 = a28; a28 = o_add(t154, a49); a49 = o_sub(t154, a49); }
    { uint64_t t155 = a46; a46 = o_add(t155, a7); a7 = o_sub(t155, a7); }
    { uint64_t t156 = a4; a4 = o_add(t156, a25); a25 = o_sub(t156, a25); }
    a25 = o_shift(a25, 48);
    { uint64_t t157 = a46; a46 = o_add(t157, a4); a4 = o_sub(t157, a4); }
    { uint64_t t158 = a7; a7 = o_add(t158, a25); a25 = o_sub(t158, a25); }
    { uint64_t t159 = a22; a22 = o_add(t159, a10); a10 = o_sub(t159, a10); }
    { uint64_t t160 = a13; a13 = o_add(t160, a43); a43 = o_sub(t160, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t161 = a22; a22 = o_add(t161, a13); a13 = o_sub(t161, a13); }
    { uint64_t t162 = a10; a10 = o_add(t162, a43); a43 = o_sub(t162, a43); }
    uint64_t t163 = a34;
    a34 = o_add(a34, a37);
    a37 = o_mul(a37, 1152921504338411520ULL);
    a31 = o_mul(a31, 6259776822214049175ULL);
    a46 = o_mul(a46, 9380094172986290191ULL);
    a22 = o_mul(a22, 891943630314919127ULL);
    a40 = o_mul(a40, 17228171707553225791ULL);
    a28 = o_mul(a28, 12855743360534130886ULL);
    a7 = o_mul(a7, 6167687396920564837ULL);
    a10 = o_mul(a10, 17201834061724655524ULL);
    a1 = o_mul(a1, 15308299771656910737ULL);
    a16 = o_mul(a16, 18186005861103657533ULL);
    a4 = o_mul(a4, 53595491891823545ULL);
    a13 = o_mul(a13, 1906638201581172103ULL);
    a19 = o_mul(a19, 18303651001328874822ULL);
    a49 = o_mul(a49, 3077466521755967626ULL);
    a25 = o_mul(a25, 12423593102987598328ULL);
    a43 = o_mul(a43, 18361513053649472048ULL);
    a37 = o_add(a37, t163);
    { uint64_t t164 = a37; a37 = o_add(t164, a1); a1 = o_sub(t164, a1); }
    { uint64_t t165 = a19; a19 = o_add(t165, a40); a40 = o_sub(t165, a40); }
    a40 = o_shift(a40, 48);
    { uint64_t t166 = a37; a37 = o_add(t166, a19); a19 = o_sub(t166, a19); }
    { uint64_t t167 = a1; a1 = o_add(t167, a40); a40 = o_sub(t167, a40); }
    { uint64_t t168 = a43; a43 = o_add(t168, a10); a10 = o_sub(t168, a10); }
    { uint64_t t169 = a13; a13 = o_add(t169, a22); a22 = o_sub(t169, a22); }
    a22 = o_shift(a22, 48);
    { uint64_t t170 = a43; a43 = o_add(t170, a13); a13 = o_sub(t170, a13); }
    { uint64_t t171 = a10; a10 = o_add(t171, a22); a22 = o_sub(t171, a22); }
    { uint64_t t172 = a25; a25 = o_add(t172, a7); a7 = o_sub(t172, a7); }
    { uint64_t t173 = a4; a4 = o_add(t173, a46); a46 = o_sub(t173, a46); }
    a46 = o_shift(a46, 48);
    { uint64_t t174 = a25; a25 = o_add(t174, a4); a4 = o_sub(t174, a4); }
    { uint64_t t175 = a7; a7 = o_add(t175, a46); a46 = o_sub(t175, a46); }
    { uint64_t t176 = a49; a49 = o_add(t176, a28); a28 = o_sub(t176, a28); }
    { uint64_t t177 = a16; a16 = o_add(t177, a31); a31 = o_sub(t177, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t178 = a49; a49 = o_add(t178, a16); a16 = o_sub(t178, a16); }
    { uint64_t t179 = a28; a28 = o_add(t179, a31); a31 = o_sub(t179, a31); }
    a10 = o_shift(a10, 12);
    a13 = o_shift(a13, 24);
    a22 = o_shift(a22, 36);
    a7 = o_shift(a7, 24);
    a4 = o_shift(a4, 48);
    a46 = o_shift(a46, 72);
    a28 = o_shift(a28, 36);
    a16 = o_shift(a16, 72);
    a31 = o_neg(o_shift(a31, 12));
    { uint64_t t180 = a37; a37 = o_add(t180, a25); a25 = o_sub(t180, a25); }
    { uint64_t t181 = a43; a43 = o_add(t181, a49); a49 = o_sub(t181, a49); }
    a49 = o_shift(a49, 48);
    { uint64_t t182 = a37; a37 = o_add(t182, a43); a43 = o_sub(t182, a43); }
    { uint64_t t183 = a25; a25 = o_add(t183, a49); a49 = o_sub(t183, a49); }
    { uint64_t t184 = a1; a1 = o_add(t184, a7); a7 = o_sub(t184, a7); }
    { uint64_t t185 = a10; a10 = o_add(t185, a28); a28 = o_sub(t185, a28); }
    a28 = o_shift(a28, 48);
    { uint64_t t186 = a1; a1 = o_add(t186, a10); a10 = o_sub(t186, a10); }
    { uint64_t t187 = a7; a7 = o_add(t187, a28); a28 = o_sub(t187, a28); }
    { uint64_t t188 = a19; a19 = o_add(t188, a4); a4 = o_sub(t188, a4); }
    { uint64_t t189 = a13; a13 = o_add(t189, a16); a16 = o_sub(t189, a16); }
    a16 = o_shift(a16, 48);
    { uint64_t t190 = a19; a19 = o_add(t190, a13); a13 = o_sub(t190, a13); }
    { uint64_t t191 = a4; a4 = o_add(t191, a16); a16 = o_sub(t191, a16); }
    { uint64_t t192 = a40; a40 = o_add(t192, a46); a46 = o_sub(t192, a46); }
    { uint64_t t193 = a22; a22 = o_add(t193, a31); a31 = o_sub(t193, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t194 = a40; a40 = o_add(t194, a22); a22 = o_sub(t194, a22); }
    { uint64_t t195 = a46; a46 = o_add(t195, a31); a31 = o_sub(t195, a31); }
    { uint64_t t196 = a0, t197 = a17, t198 = a34;
      a0 = o_add(o_add(t196, t197), t198);
      a17 = o_sub(o_add(t196, o_shift(t197, 64)), o_shift(t198, 32));
      a34 = o_add(o_sub(t196, o_shift(t197, 32)), o_shift(t198, 64)); }
    { uint64_t t199 = a3, t200 = a20, t201 = a37;
      a3 = o_add(o_add(t199, t200), t201);
      a20 = o_sub(o_add(t199, o_shift(t200, 64)), o_shift(t201, 32));
      a37 = o_add(o_sub(t199, o_shift(t200, 32)), o_shift(t201, 64)); }
    { uint64_t t202 = a33, t203 = a50, t204 = a16;
      a33 = o_add(o_add(t202, t203), t204);
      a50 = o_sub(o_add(t202, o_shift(t203, 64)), o_shift(t204, 32));
      a16 = o_add(o_sub(t202, o_shift(t203, 32)), o_shift(t204, 64)); }
    { uint64_t t205 = a18, t206 = a35, t207 = a1;
      a18 = o_add(o_add(t205, t206), t207);
      a35 = o_sub(o_add(t205, o_shift(t206, 64)), o_shift(t207, 32));
      a1 = o_add(o_sub(t205, o_shift(t206, 32)), o_shift(t207, 64)); }
    { uint64_t t208 = a15, t209 = a32, t210 = a49;
      a15 = o_add(o_add(t208, t209), t210);
      a32 = o_sub(o_add(t208, o_shift(t209, 64)), o_shift(t210, 32));
      a49 = o_add(o_sub(t208, o_shift(t209, 32)), o_shift(t210, 64)); }
    { uint64_t t211 = a24, t212 = a41, t213 = a7;
      a24 = o_add(o_add(t211, t212), t213);
      a41 = o_sub(o_add(t211, o_shift(t212, 64)), o_shift(t213, 32));
      a7 = o_add(o_sub(t211, o_shift(t212, 32)), o_shift(t213, 64)); }
    { uint64_t t214 = a48, t215 = a14, t216 = a31;
      a48 = o_add(o_add(t214, t215), t216);
      a14 = o_sub(o_add(t214, o_shift(t215, 64)), o_shift(t216, 32));
      a31 = o_add(o_sub(t214, o_shift(t215, 32)), o_shift(t216, 64)); }
    { uint64_t t217 = a39, t218 = a5, t219 = a22;
      a39 = o_add(o_add(t217, t218), t219);
      a5 = o_sub(o_add(t217, o_shift(t218, 64)), o_shift(t219, 32));
      a22 = o_add(o_sub(t217, o_shift(t218, 32)), o_shift(t219, 64)); }
    { uint64_t t220 = a30, t221 = a47, t222 = a13;
      a30 = o_add(o_add(t220, t221), t222);
      a47 = o_sub(o_add(t220, o_shift(t221, 64)), o_shift(t222, 32));
      a13 = o_add(o_sub(t220, o_shift(t221, 32)), o_shift(t222, 64)); }
    { uint64_t t223 = a36, t224 = a2, t225 = a19;
      a36 = o_add(o_add(t223, t224), t225);
      a2 = o_sub(o_add(t223, o_shift(t224, 64)), o_shift(t225, 32));
      a19 = o_add(o_sub(t223, o_shift(t224, 32)), o_shift(t225, 64)); }
    { uint64_t t226 = a6, t227 = a23, t228 = a40;
      a6 = o_add(o_add(t226, t227), t228);
      a23 = o_sub(o_add(t226, o_shift(t227, 64)), o_shift(t228, 32));
      a40 = o_add(o_sub(t226, o_shift(t227, 32)), o_shift(t228, 64)); }
    { uint64_t t229 = a12, t230 = a29, t231 = a46;
      a12 = o_add(o_add(t229, t230), t231);
      a29 = o_sub(o_add(t229, o_shift(t230, 64)), o_shift(t231, 32));
      a46 = o_add(o_sub(t229, o_shift(t230, 32)), o_shift(t231, 64)); }
    { uint64_t t232 = a45, t233 = a11, t234 = a28;
      a45 = o_add(o_add(t232, t233), t234);
      a11 = o_sub(o_add(t232, o_shift(t233, 64)), o_shift(t234, 32));
      a28 = o_add(o_sub(t232, o_shift(t233, 32)), o_shift(t234, 64)); }
    { uint64_t t235 = a42, t236 = a8, t237 = a25;
      a42 = o_add(o_add(t235, t236), t237);
      a8 = o_sub(o_add(t235, o_shift(t236, 64)), o_shift(t237, 32));
      a25 = o_add(o_sub(t235, o_shift(t236, 32)), o_shift(t237, 64)); }
    { uint64_t t238 = a27, t239 = a44, t240 = a10;
      a27 = o_add(o_add(t238, t239), t240);
      a44 = o_sub(o_add(t238, o_shift(t239, 64)), o_shift(t240, 32));
      a10 = o_add(o_sub(t238, o_shift(t239, 32)), o_shift(t240, 64)); }
    { uint64_t t241 = a21, t242 = a38, t243 = a4;
      a21 = o_add(o_add(t241, t242), t243);
      a38 = o_sub(o_add(t241, o_shift(t242, 64)), o_shift(t243, 32));
      a4 = o_add(o_sub(t241, o_shift(t242, 32)), o_shift(t243, 64)); }
    { uint64_t t244 = a9, t245 = a26, t246 = a43;
      a9 = o_add(o_add(t244, t245), t246);
      a26 = o_sub(o_add(t244, o_shift(t245, 64)), o_shift(t246, 32));
      a43 = o_add(o_sub(t244, o_shift(t245, 32)), o_shift(t246, 64)); }
    v[0] = a0;
    v[1] = a20;
    v[2] = a16;
    v[3] = a18;
    v[4] = a32;
    v[5] = a7;
    v[6] = a48;
    v[7] = a5;
    v[8] = a13;
    v[9] = a36;
    v[10] = a23;
    v[11] = a46;
    v[12] = a45;
    v[13] = a8;
    v[14] = a10;
    v[15] = a21;
    v[16] = a26;
    v[17] = a34;
    v[18] = a3;
    v[19] = a50;
    v[20] = a1;
    v[21] = a15;
    v[22] = a41;
    v[23] = a31;
    v[24] = a39;
    v[25] = a47;
    v[26] = a19;
    v[27] = a6;
    v[28] = a29;
    v[29] = a28;
    v[30] = a42;
    v[31] = a44;
    v[32] = a4;
    v[33] = a9;
    v[34] = a17;
    v[35] = a37;
    v[36] = a33;
    v[37] = a35;
    v[38] = a49;
    v[39] = a24;
    v[40] = a14;
    v[41] = a22;
    v[42] = a30;
    v[43] = a2;
    v[44] = a40;
    v[45] = a12;
    v[46] = a11;
    v[47] = a25;
    v[48] = a27;
    v[49] = a38;
    v[50] = a43;
}

static void o_ntt_60(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33], a34 = v[34], a35 = v[35], a36 = v[36], a37 = v[37], a38 = v[38], a39 = v[39], a40 = v[40], a41 = v[41], a42 = v[42], a43 = v[43], a44 = v[44], a45 = v[45], a46 = v[46], a47 = v[47], a48 = v[48], a49 = v[49], a50 = v[50], a51 = v[51], a52 = v[52], a53 = v[53], a54 = v[54], a55 = v[55], a56 = v[56], a57 = v[57], a58 = v[58], a59 = v[59];
    { uint64_t t1 = a0, t2 = a20, t3 = a40;
      a0 = o_add(o_add(t1, t2), t3);
      a20 = o_sub(o_add(t1, o_shift(t2, 64)), o_shift(t3, 32));
      a40 = o_add(o_sub(t1, o_shift(t2, 32)), o_shift(t3, 64)); }
    { uint64_t t4 = a30, t5 = a50, t6 = a10;
      a30 = o_add(o_add(t4, t5), t6);
      a50 = o_sub(o_add(t4, o_shift(t5, 64)), o_shift(t6, 32));
      a10 = o_add(o_sub(t4, o_shift(t5, 32)), o_shift(t6, 64)); }
    { uint64_t t7 = a0; a0 = o_add(t7, a30); a30 = o_sub(t7, a30); }
    { uint64_t t8 = a20; a20 = o_add(t8, a50); a50 = o_sub(t8, a50); }
    { uint64_t t9 = a40; a40 = o_add(t9, a10); a10 = o_sub(t9, a10); }
    { uint64_t t10 = a1, t11 = a21, t12 = a41;
      a1 = o_add(o_add(t10, t11), t12);
      a21 = o_sub(o_add(t10, o_shift(t11, 64)), o_shift(t12, 32));
      a41 = o_add(o_sub(t10, o_shift(t11, 32)), o_shift(t12, 64)); }
    { uint64_t t13 = a31, t14 = a51, t15 = a11;
      a31 = o_add(o_add(t13, t14), t15);
      a51 = o_sub(o_add(t13, o_shift(t14, 64)), o_shift(t15, 32));
      a11 = o_add(o_sub(t13, o_shift(t14, 32)), o_shift(t15, 64)); }
    { uint64_t t16 = a1; a1 = o_add(t16, a31); a31 = o_sub(t16, a31); }
    { uint64_t t17 = a21; a21 = o_add(t17, a51); a51 = o_sub(t17, a51); }
    { uint64_t t18 = a41; a41 = o_add(t18, a11); a11 = o_sub(t18, a11); }
    { uint64_t t19 = a2, t20 = a22, t21 = a42;
      a2 = o_add(o_add(t19, t20), t21);
      a22 = o_sub(o_add(t19, o_shift(t20, 64)), o_shift(t21, 32));
      a42 = o_add(o_sub(t19, o_shift(t20, 32)), o_shift(t21, 64)); }
    { uint64_t t22 = a32, t23 = a52, t24 = a12;
      a32 = o_add(o_add(t22, t23), t24);
      a52 = o_sub(o_add(t22, o_shift(t23, 64)), o_shift(t24, 32));
      a12 = o_add(o_sub(t22, o_shift(t23, 32)), o_shift(t24, 64)); }
    { uint64_t t25 = a2; a2 = o_add(t25, a32); a32 = o_sub(t25, a32); }
    { uint64_t t26 = a22; a22 = o_add(t26, a52); a52 = o_sub(t26, a52); }
    { uint64_t t27 = a42; a42 = o_add(t27, a12); a12 = o_sub(t27, a12); }
    { uint64_t t28 = a3, t29 = a23, t30 = a43;
      a3 = o_add(o_add(t28, t29), t30);
      a23 = o_sub(o_add(t28, o_shift(t29, 64)), o_shift(t30, 32));
      a43 = o_add(o_sub(t28, o_shift(t29, 32)), o_shift(t30, 64)); }
    { uint64_t t31 = a33, t32 = a53, t33 = a13;
      a33 = o_add(o_add(t31, t32), t33);
      a53 = o_sub(o_add(t31, o_shift(t32, 64)), o_shift(t33, 32));
      a13 = o_add(o_sub(t31, o_shift(t32, 32)), o_shift(t33, 64)); }
    { uint64_t t34 = a3; a3 = o_add(t34, a33); a33 = o_sub(t34, a33); }
    { uint64_t t35 = a23; a23 = o_add(t35, a53); a53 = o_sub(t35, a53); }
    { uint64_t t36 = a43; a43 = o_add(t36, a13); a13 = o_sub(t36, a13); }
    { uint64_t t37 = a4, t38 = a24, t39 = a44;
      a4 = o_add(o_add(t37, t38), t39);
      a24 = o_sub(o_add(t37, o_shift(t38, 64)), o_shift(t39, 32));
      a44 = o_add(o_sub(t37, o_shift(t38, 32)), o_shift(t39, 64)); }
    { uint64_t t40 = a34, t41 = a54, t42 = a14;
      a34 = o_add(o_add(t40, t41), t42);
      a54 = o_sub(o_add(t40, o_shift(t41, 64)), o_shift(t42, 32));
      a14 = o_add(o_sub(t40, o_shift(t41, 32)), o_shift(t42, 64)); }
    { uint64_t t43 = a4; a4 = o_add(t43, a34); a34 = o_sub(t43, a34); }
    { uint64_t t44 = a24; a24 = o_add(t44, a54); a54 = o_sub(t44, a54); }
    { uint64_t t45 = a44; a44 = o_add(t45, a14); a14 = o_sub(t45, a14); }
    { uint64_t t46 = a5, t47 = a25, t48 = a45;
      a5 = o_add(o_add(t46, t47), t48);
      a25 = o_sub(o_add(t46, o_shift(t47, 64)), o_shift(t48, 32));
      a45 = o_add(o_sub(t46, o_shift(t47, 32)), o_shift(t48, 64)); }
    { uint64_t t49 = a35, t50 = a55, t51 = a15;
      a35 = o_add(o_add(t49, t50), t51);
      a55 = o_sub(o_add(t49, o_shift(t50, 64)), o_shift(t51, 32));
      a15 = o_add(o_sub(t49, o_shift(t50, 32)), o_shift(t51, 64)); }
    { uint64_t t52 = a5; a5 = o_add(t52, a35); a35 = o_sub(t52, a35); }
    { uint64_t t53 = a25; a25 = o_add(t53, a55); a55 = o_sub(t53, a55); }
    { uint64_t t54 = a45; a45 = o_add(t54, a15); a15 = o_sub(t54, a15); }
    { uint64_t t55 = a6, t56 = a26, t57 = a46;
      a6 = o_add(o_add(t55, t56), t57);
      a26 = o_sub(o_add(t55, o_shift(t56, 64)), o_shift(t57, 32));
      a46 = o_add(o_sub(t55, o_shift(t56, 32)), o_shift(t57, 64)); }
    { uint64_t t58 = a36, t59 = a56, t60 = a16;
      a36 = o_add(o_add(t58, t59), t60);
      a56 = o_sub(o_add(t58, o_shift(t59, 64)), o_shift(t60, 32));
      a16 = o_add(o_sub(t58, o_shift(t59, 32)), o_shift(t60, 64)); }
    { uint64_t t61 = a6; a6 = o_add(t61, a36); a36 = o_sub(t61, a36); }
    { uint64_t t62 = a26; a26 = o_add(t62, a56); a56 = o_sub(t62, a56); }
    { uint64_t t63 = a46; a46 = o_add(t63, a16); a16 = o_sub(t63, a16); }
    { uint64_t t64 = a7, t65 = a27, t66 = a47;
      a7 = o_add(o_add(t64, t65), t66);
      a27 = o_sub(o_add(t64, o_shift(t65, 64)), o_shift(t66, 32));
      a47 = o_add(o_sub(t64, o_shift(t65, 32)), o_shift(t66, 64)); }
    { uint64_t t67 = a37, t68 = a57, t69 = a17;
      a37 = o_add(o_add(t67, t68), t69);
      a57 = o_sub(o_add(t67, o_shift(t68, 64)), o_shift(t69, 32));
      a17 = o_add(o_sub(t67, o_shift(t68, 32)), o_shift(t69, 64)); }
    { uint64_t t70 = a7; a7 = o_add(t70, a37); a37 = o_sub(t70, a37); }
    { uint64_t t71 = a27; a27 = o_add(t71, a57); a57 = o_sub(t71, a57); }
    { uint64_t t72 = a47; a47 = o_add(t72, a17); a17 = o_sub(t72, a17); }
    { uint64_t t73 = a8, t74 = a28, t75 = a48;
      a8 = o_add(o_add(t73, t74), t75);
      a28 = o_sub(o_add(t73, o_shift(t74, 64)), o_shift(t75, 32));
      a48 = o_add(o_sub(t73, o_shift(t74, 32)), o_shift(t75, 64)); }
    { uint64_t t76 = a38, t77 = a58, t78 = a18;
      a38 = o_add(o_add(t76, t77), t78);
      a58 = o_sub(o_add(t76, o_shift(t77, 64)), o_shift(t78, 32));
      a18 = o_add(o_sub(t76, o_shift(t77, 32)), o_shift(t78, 64)); }
    { uint64_t t79 = a8; a8 = o_add(t79, a38); a38 = o_sub(t79, a38); }
    { uint64_t t80 = a28; a28 = o_add(t80, a58); a58 = o_sub(t80, a58); }
    { uint64_t t81 = a48; a48 = o_add(t81, a18); a18 = o_sub(t81, a18); }
    { uint64_t t82 = a9, t83 = a29, t84 = a49;
      a9 = o_add(o_add(t82, t83), t84);
      a29 = o_sub(o_add(t82, o_shift(t83, 64)), o_shift(t84, 32));
      a49 = o_add(o_sub(t82, o_shift(t83, 32)), o_shift(t84, 64)); }
    { uint64_t t85 = a39, t86 = a59, t87 = a19;
      a39 = o_add(o_add(t85, t86), t87);
      a59 = o_sub(o_add(t85, o_shift(t86, 64)), o_shift(t87, 32));
      a19 = o_add(o_sub(t85, o_shift(t86, 32)), o_shift(t87, 64)); }
    { uint64_t t88 = a9; a9 = o_add(t88, a39); a39 = o_sub(t88, a39); }
    { uint64_t t89 = a29; a29 = o_add(t89, a59); a59 = o_sub(t89, a59); }
    { uint64_t t90 = a49; a49 = o_add(t90, a19); a19 = o_sub(t90, a19); }
    a51 = o_mul(a51, 5927015354646419725ULL);
    a41 = o_mul(a41, 6868348408044855211ULL);
    a31 = o_mul(a31, 5290193119087387221ULL);
    a21 = o_mul(a21, 17775832080808074370ULL);
    a11 = o_shift(a11, 16);
    a52 = o_mul(a52, 6868348408044855211ULL);
    a42 = o_mul(a42, 17775832080808074370ULL);
    a32 = o_mul(a32, 18235156514275634624ULL);
    a22 = o_mul(a22, 9988211933311186582ULL);
    a12 = o_shift(a12, 32);
    a53 = o_mul(a53, 5290193119087387221ULL);
    a43 = o_mul(a43, 18235156514275634624ULL);
    a33 = o_mul(a33, 8149776168132872528ULL);
    a23 = o_mul(a23, 1041288259238279555ULL);
    a13 = o_shift(a13, 48);
    a54 = o_mul(a54, 17775832080808074370ULL);
    a44 = o_mul(a44, 9988211933311186582ULL);
    a34 = o_mul(a34, 1041288259238279555ULL);
    a24 = o_mul(a24, 6205107048362784195ULL);
    a14 = o_shift(a14, 64);
    a55 = o_shift(a55, 16);
    a45 = o_shift(a45, 32);
    a35 = o_shift(a35, 48);
    a25 = o_shift(a25, 64);
    a15 = o_shift(a15, 80);
    a56 = o_mul(a56, 18235156514275634624ULL);
    a46 = o_mul(a46, 1041288259238279555ULL);
    a36 = o_mul(a36, 17073700798457888299ULL);
    a26 = o_mul(a26, 15820824984080659046ULL);
    a16 = o_neg(a16);
    a57 = o_mul(a57, 5079231842359091375ULL);
    a47 = o_mul(a47, 15149912995474149095ULL);
    a37 = o_mul(a37, 17869255328328231396ULL);
    a27 = o_mul(a27, 7085488865146701717ULL);
    a17 = o_neg(o_shift(a17, 16));
    a58 = o_mul(a58, 9988211933311186582ULL);
    a48 = o_mul(a48, 6205107048362784195ULL);
    a38 = o_mul(a38, 15820824984080659046ULL);
    a28 = o_mul(a28, 11578395661369729110ULL);
    a18 = o_neg(o_shift(a18, 32));
    a59 = o_mul(a59, 8149776168132872528ULL);
    a49 = o_mul(a49, 17073700798457888299ULL);
    a39 = o_mul(a39, 2281812832982421726ULL);
    a29 = o_mul(a29, 211587555138949697ULL);
    a19 = o_neg(o_shift(a19, 48));
    { uint64_t t91 = a2; a2 = o_add(t91, a8); a8 = o_sub(t91, a8); }
    { uint64_t t92 = a6; a6 = o_add(t92, a4); a4 = o_sub(t92, a4); }
    a4 = o_shift(a4, 48);
    { uint64_t t93 = a2; a2 = o_add(t93, a6); a6 = o_sub(t93, a6); }
    { uint64_t t94 = a8; a8 = o_add(t94, a4); a4 = o_sub(t94, a4); }
    uint64_t t95 = a0;
    a0 = o_add(a0, a2);
    a2 = o_mul(a2, 4611686017353646080ULL);
    a8 = o_mul(a8, 16181989089180173841ULL);
    a6 = o_mul(a6, 5818851782451133869ULL);
    a4 = o_mul(a4, 11322249509082494407ULL);
    a2 = o_add(a2, t95);
    { uint64_t t96 = a2; a2 = o_add(t96, a6); a6 = o_sub(t96, a6); }
    { uint64_t t97 = a4; a4 = o_add(t97, a8); a8 = o_sub(t97, a8); }
    a8 = o_shift(a8, 48);
    { uint64_t t98 = a2; a2 = o_add(t98, a4); a4 = o_sub(t98, a4); }
    { uint64_t t99 = a6; a6 = o_add(t99, a8); a8 = o_sub(t99, a8); }
    { uint64_t t100 = a7; a7 = o_add(t100, a3); a3 = o_sub(t100, a3); }
    { uint64_t t101 = a1; a1 = o_add(t101, a9); a9 = o_sub(t101, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t102 = a7; a7 = o_add(t102, a1); a1 = o_sub(t102, a1); }
    { uint64_t t103 = a3; a3 = o_add(t103, a9); a9 = o_sub(t103, a9); }
    uint64_t t104 = a5;
    a5 = o_add(a5, a7);
    a7 = o_mul(a7, 4611686017353646080ULL);
    a3 = o_mul(a3, 16181989089180173841ULL);
    a1 = o_mul(a1, 5818851782451133869ULL);
    a9 = o_mul(a9, 11322249509082494407ULL);
    a7 = o_add(a7, t104);
    { uint64_t t105 = a7; a7 = o_add(t105, a1); a1 = o_sub(t105, a1); }
    { uint64_t t106 = a9; a9 = o_add(t106, a3); a3 = o_sub(t106, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t107 = a7; a7 = o_add(t107, a9); a9 = o_sub(t107, a9); }
    { uint64_t t108 = a1; a1 = o_add(t108, a3); a3 = o_sub(t108, a3); }
    { uint64_t t109 = a0; a0 = o_add(t109, a5); a5 = o_sub(t109, a5); }
    { uint64_t t110 = a2; a2 = o_add(t110, a7); a7 = o_sub(t110, a7); }
    { uint64_t t111 = a6; a6 = o_add(t111, a1); a1 = o_sub(t111, a1); }
    { uint64_t t112 = a8; a8 = o_add(t112, a3); a3 = o_sub(t112, a3); }
    { uint64_t t113 = a4; a4 = o_add(t113, a9); a9 = o_sub(t113, a9); }
    { uint64_t t114 = a52; a52 = o_add(t114, a58); a58 = o_sub(t114, a58); }
    { uint64_t t115 = a56; a56 = o_add(t115, a54); a54 = o_sub(t115, a54); }
    a54 = o_shift(a54, 48);
    { uint64_t t116 = a52; a52 = o_add(t116, a56); a56 = o_sub(t116, a56); }
    { uint64_t t117 = a58; a58 = o_add(t117, a54); a54 = o_sub(t117, a54); }
    uint64_t t118 = a50;
    a50 = o_add(a50, a52);
    a52 = o_mul(a52, 4611686017353646080ULL);
    a58 = o_mul(a58, 16181989089180173841ULL);
    a56 = o_mul(a56, 5818851782451133869ULL);
    a54 = o_mul(a54, 11322249509082494407ULL);
    a52 = o_add(a52, t118);
    { uint64_t t119 = a52; a52 = o_add(t119, a56); a56 = o_sub(t119, a56); }
    { uint64_t t120 = a54; a54 = o_add(t120, a58); a58 = o_sub(t120, a58); }
    a58 = o_shift(a58, 48);
    { uint64_t t121 = a52; a52 = o_add(t121, a54); a54 = o_sub(t121, a54); }
    { uint64_t t122 = a56; a56 = o_add(t122, a58); a58 = o_sub(t122, a58); }
    { uint64_t t123 = a57; a57 = o_add(t123, a53); a53 = o_sub(t123, a53); }
    { uint64_t t124 = a51; a51 = o_add(t124, a59); a59 = o_sub(t124, a59); }
    a59 = o_shift(a59, 48);
    { uint64_t t125 = a57; a57 = o_add(t125, a51); a51 = o_sub(t125, a51); }
    { uint64_t t126 = a53; a53 = o_add(t126, a59); a59 = o_sub(t126, a59); }
    uint64_t t127 = a55;
    a55 = o_add(a55, a57);
    a57 = o_mul(a57, 4611686017353646080ULL);
    a53 = o_mul(a53, 16181989089180173841ULL);
    a51 = o_mul(a51, 5818851782451133869ULL);
    a59 = o_mul(a59, 11322249509082494407ULL);
    a57 = o_add(a57, t127);
    { uint64_t t128 = a57; a57 = o_add(t128, a51); a51 = o_sub(t128, a51); }
    { uint64_t t129 = a59; a59 = o_add(t129, a53); a53 = o_sub(t129, a53); }
    a53 = o_shift(a53, 48);
    { uint64_t t130 = a57; a57 = o_add(t130, a59); a59 = o_sub(t130, a59); }
    { uint64_t t131 = a51; a51 = o_add(t131, a53); a53 = o_sub(t131, a53); }
    { uint64_t t132 = a50; a50 = o_add(t132, a55); a55 = o_sub(t132, a55); }
    { uint64_t t133 = a52; a52 = o_add(t133, a57); a57 = o_sub(t133, a57); }
    { uint64_t t134 = a56; a56 = o_add(t134, a51); a51 = o_sub(t134, a51); }
    { uint64_t t135 = a58; a58 = o_add(t135, a53); a53 = o_sub(t135, a53); }
    { uint64_t t136 = a54; a54 = o_add(t136, a59); a59 = o_sub(t136, a59); }
    { uint64_t t137 = a42; a42 = o_add(t137, a48); a48 = o_sub(t137, a48); }
    { uint64_t t138 = a46; a46 = o_add(t138, a44); a44 = o_sub(t138, a44); }
    a44 = o_shift(a44, 48);
    { uint64_t t139 = a42; a42 = o_add(t139, a46); a46 = o_sub(t139, a46); }
    { uint64_t t140 = a48; a48 = o_add(t140, a44); a44 = o_sub(t140, a44); }
    uint64_t t141 = a40;
    a40 = o_add(a40, a42);
    a42 = o_mul(a42, 4611686017353646080ULL);
    a48 = o_mul(a48, 16181989089180173841ULL);
    a46 = o_mul(a46, 5818851782451133869ULL);
    a44 = o_mul(a44, 11322249509082494407ULL);
    a42 = o_add(a42, t141);
    { uint64_t t142 = a42; a42 = o_add(t142, a46); a46 = o_sub(t142, a46); }
    { uint64_t t143 = a44; a44 = o_add(t143, a48); a48 = o_sub(t143, a48); }
    a48 = o_shift(a48, 48);
    { uint64_t t144 = a42; a42 = o_add(t144, a44); a44 = o_sub(t144, a44); }
    { uint64_t t145 = a46; a46 = o_add(t145, a48); a48 = o_sub(t145, a48); }
    { uint64_t t146 = a47; a47 = o_add(t146, a43); a43 = o_sub(t146, a43); }
    { uint64_t t147 = a41; a41 = o_add(t147, a49); a49 = o_sub(t147, a49); }
    a49 = o_shift(a49, 48);
    { uint64_t t148 = a47; a47 = o_add(t148, a41); a41 = o_sub(t148, a41); }
    { uint64_t t149 = a43; a43 = o_add(t149, a49); a49 = o_sub(t149, a49); }
    uint64_t t150 = a45;
    a45 = o_add(a45, a47);
    a47 = o_mul(a47, 4611686017353646080ULL);
    a43 = o_mul(a43, 16181989089180173841ULL);
    a41 = o_mul(a41, 5818851782451133869ULL);
    a49 = o_mul(a49, 11322249509082494407ULL);
    a47 = o_add(a47, t150);
    { uint64_t t151 = a47; a47 = o_add(t151, a41); a41 = o_sub(t151, a41); }
    { uint64_t t152 = a49; a49 = o_add(t152, a43); a43 = o_sub(t152, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t153 = a47; a47 = o_add(t153, a49); a49 = o_sub(t153, a49); }
    { uint64_t t154 = a41; a41 = o_add(t154, a43); a43 = o_sub(t154, a43); }
    { uint64_t t155 = a40; a40 = o_add(t155, a45); a45 = o_sub(t155, a45); }
    { uint64_t t156 = a42; a42 = o_add(t156, a47); a47 = o_sub(t156, a47); }
    { uint64_t t157 = a46; a46 = o_add(t157, a41); a41 = o_sub(t157, a41); }
    { uint64_t t158 = a48; a48 = o_add(t158, a43); a43 = o_sub(t158, a43); }
    { uint64_t t159 = a44; a44 = o_add(t159, a49); a49 = o_sub(t159, a49); }
    { uint64_t t160 = a32; a32 = o_add(t160, a38); a38 = o_sub(t160, a38); }
    { uint64_t t161 = a36; a36 = o_add(t161, a34); a34 = o_sub(t161, a34); }
    a34 = o_shift(a34, 48);
    { uint64_t t162 = a32; a32 = o_add(t162, a36); a36 = o_sub(t162, a36); }
    { uint64_t t163 = a38; a38 = o_add(t163, a34); a34 = o_sub(t163, a34); }
    uint64_t t164 = a30;
    a30 = o_add(a30, a32);
    a32 = o_mul(a32, 4611686017353646080ULL);
    a38 = o_mul(a38, 16181989089180173841ULL);
    a36 = o_mul(a36, 5818851782451133869ULL);
    a34 = o_mul(a34, 11322249509082494407ULL);
    a32 = o_add(a32, t164);
    { uint64_t t165 = a32; a32 = o_add(t165, a36); a36 = o_sub(t165, a36); }
    { uint64_t t166 = a34; a34 = o_add(t166, a38); a38 = o_sub(t166, a38); }
    a38 = o_shift(a38, 48);
    { uint64_t t167 = a32; a32 = o_add(t167, a34); a34 = o_sub(t167, a34); }
    { uint64_t t168 = a36; a36 = o_add(t168, a38); a38 = o_sub(t168, a38); }
    { uint64_t t169 = a37; a37 = o_add(t169, a33); a33 = o_sub(t169, a33); }
    { uint64_t t170 = a31; a31 = o_add(t170, a39); a39 = o_sub(t170, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t171 = a37; a37 = o_add(t171, a31); a31 = o_sub(t171, a31); }
    { uint64_t t172 = a33; a33 = o_add(t172, a39); a39 = o_sub(t172, a39); }
    uint64_t t173 = a35;
    a35 = o_add(a35, a37);
    a37 = o_mul(a37, 4611686017353646080ULL);
    a33 = o_mul(a33, 16181989089180173841ULL);
    a31 = o_mul(a31, 5818851782451133869ULL);
    a39 = o_mul(a39, 11322249509082494407ULL);
    a37 = o_add(a37, t173);
    { uint64_t t174 = a37; a37 = o_add(t174, a31); a31 = o_sub(t174, a31); }
    { uint64_t t175 = a39; a39 = o_add(t175, a33); a33 = o_sub(t175, a33); }
    a33 = o_shift(a33, 48);
    { uint64_t t176 = a37; a37 = o_add(t176, a39); a39 = o_sub(t176, a39); }
    { uint64_t t177 = a31; a31 = o_add(t177, a33); a33 = o_sub(t177, a33); }
    { uint64_t t178 = a30; a30 = o_add(t178, a35); a35 = o_sub(t178, a35); }
    { uint64_t t179 = a32; a32 = o_add(t179, a37); a37 = o_sub(t179, a37); }
    { uint64_t t180 = a36; a36 = o_add(t180, a31); a31 = o_sub(t180, a31); }
    { uint64_t t181 = a38; a38 = o_add(t181, a33); a33 = o_sub(t181, a33); }
    { uint64_t t182 = a34; a34 = o_add(t182, a39); a39 = o_sub(t182, a39); }
    { uint64_t t183 = a22; a22 = o_add(t183, a28); a28 = o_sub(t183, a28); }
    { uint64_t t184 = a26; a26 = o_add(t184, a24); a24 = o_sub(t184, a24); }
    a24 = o_shift(a24, 48);
    { uint64_t t185 = a22; a22 = o_add(t185, a26); a26 = o_sub(t185, a26); }
    { uint64_t t186 = a28; a28 = o_add(t186, a24); a24 = o_sub(t186, a24); }
    uint64_t t187 = a20;
    a20 = o_add(a20, a22);
    a22 = o_mul(a22, 4611686017353646080ULL);
    a28 = o_mul(a28, 16181989089180173841ULL);
    a26 = o_mul(a26, 5818851782451133869ULL);
    a24 = o_mul(a24, 11322249509082494407ULL);
    a22 = o_add(a22, t187);
    { uint64_t t188 = a22; a22 = o_add(t188, a26); a26 = o_sub(t188, a26); }
    { uint64_t t189 = a24; a24 = o_add(t189, a28); a28 = o_sub(t189, a28); }
    a28 = o_shift(a28, 48);
    { uint64_t t190 = a22; a22 = o_add(t190, a24); a24 = o_sub(t190, a24); }
    { uint64_t t191 = a26; a26 = o_add(t191, a28); a28 = o_sub(t191, a28); }
    { uint64_t t192 = a27; a27 = o_add(t192, a23); a23 = o_sub(t192, a23); }
    { uint64_t t193 = a21; a21 = o_add(t193, a29); a29 = o_sub(t193, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t194 = a27; a27 = o_add(t194, a21); a21 = o_sub(t194, a21); }
    { uint64_t t195 = a23; a23 = o_add(t195, a29); a29 = o_sub(t195, a29); }
    uint64_t t196 = a25;
    a25 = o_add(a25, a27);
    a27 = o_mul(a27, 4611686017353646080ULL);
    a23 = o_mul(a23, 16181989089180173841ULL);
    a21 = o_mul(a21, 5818851782451133869ULL);
    a29 = o_mul(a29, 11322249509082494407ULL);
    a27 = o_add(a27, t196);
    { uint64_t t197 = a27; a27 = o_add(t197, a21); a21 = o_sub(t197, a21); }
    { uint64_t t198 = a29; a29 = o_add(t198, a23); a23 = o_sub(t198, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t199 = a27; a27 = o_add(t199, a29); a29 = o_sub(t199, a29); }
    { uint64_t t200 = a21; a21 = o_add(t200, a23); a23 = o_sub(t200, a23); }
    { uint64_t t201 = a20; a20 = o_add(t201, a25); a25 = o_sub(t201, a25); }
    { uint64_t t202 = a22; a22 = o_add(t202, a27); a27 = o_sub(t202, a27); }
    { uint64_t t203 = a26; a26 = o_add(t203, a21); a21 = o_sub(t203, a21); }
    { uint64_t t204 = a28; a28 = o_add(t204, a23); a23 = o_sub(t204, a23); }
    { uint64_t t205 = a24; a24 = o_add(t205, a29); a29 = o_sub(t205, a29); }
    { uint64_t t206 = a12; a12 = o_add(t206, a18); a18 = o_sub(t206, a18); }
    { uint64_t t207 = a16; a16 = o_add(t207, a14); a14 = o_sub(t207, a14); }
    a14 = o_shift(a14, 48);
    { uint64_t t208 = a12; a12 = o_add(t208, a16); a16 = o_sub(t208, a16); }
    { uint64_t t209 = a18; a18 = o_add(t209, a14); a14 = o_sub(t209, a14); }
    uint64_t t210 = a10;
    a10 = o_add(a10, a12);
    a12 = o_mul(a12, 4611686017353646080ULL);
    a18 = o_mul(a18, 16181989089180173841ULL);
    a16 = o_mul(a16, 5818851782451133869ULL);
    a14 = o_mul(a14, 11322249509082494407ULL);
    a12 = o_add(a12, t210);
    { uint64_t t211 = a12; a12 = o_add(t211, a16); a16 = o_sub(t211, a16); }
    { uint64_t t212 = a14; a14 = o_add(t212, a18); a18 = o_sub(t212, a18); }
    a18 = o_shift(a18, 48);
    { uint64_t t213 = a12; a12 = o_add(t213, a14); a14 = o_sub(t213, a14); }
    { uint64_t t214 = a16; a16 = o_add(t214, a18); a18 = o_sub(t214, a18); }
    { uint64_t t215 = a17; a17 = o_add(t215, a13); a13 = o_sub(t215, a13); }
    { uint64_t t216 = a11; a11 = o_add(t216, a19); a19 = o_sub(t216, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t217 = a17; a17 = o_add(t217, a11); a11 = o_sub(t217, a11); }
    { uint64_t t218 = a13; a13 = o_add(t218, a19); a19 = o_sub(t218, a19); }
    uint64_t t219 = a15;
    a15 = o_add(a15, a17);
    a17 = o_mul(a17, 4611686017353646080ULL);
    a13 = o_mul(a13, 16181989089180173841ULL);
    a11 = o_mul(a11, 5818851782451133869ULL);
    a19 = o_mul(a19, 11322249509082494407ULL);
    a17 = o_add(a17, t219);
    { uint64_t t220 = a17; a17 = o_add(t220, a11); a11 = o_sub(t220, a11); }
    { uint64_t t221 = a19; a19 = o_add(t221, a13); a13 = o_sub(t221, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t222 = a17; a17 = o_add(t222, a19); a19 = o_sub(t222, a19); }
    { uint64_t t223 = a11; a11 = o_add(t223, a13); a13 = o_sub(t223, a13); }
    { uint64_t t224 = a10; a10 = o_add(t224, a15); a15 = o_sub(t224, a15); }
    { uint64_t t225 = a12; a12 = o_add(t225, a17); a17 = o_sub(t225, a17); }
    { uint64_t t226 = a16; a16 = o_add(t226, a11); a11 = o_sub(t226, a11); }
    { uint64_t t227 = a18; a18 = o_add(t227, a13); a13 = o_sub(t227, a13); }
    { uint64_t t228 = a14; a14 = o_add(t228, a19); a19 = o_sub(t228, a19); }
    v[0] = a0;
    v[1] = a50;
    v[2] = a40;
    v[3] = a30;
    v[4] = a20;
    v[5] = a10;
    v[6] = a7;
    v[7] = a57;
    v[8] = a47;
    v[9] = a37;
    v[10] = a27;
    v[11] = a17;
    v[12] = a6;
    v[13] = a56;
    v[14] = a46;
    v[15] = a36;
    v[16] = a26;
    v[17] = a16;
    v[18] = a3;
    v[19] = a53;
    v[20] = a43;
    v[21] = a33;
    v[22] = a23;
    v[23] = a13;
    v[24] = a4;
    v[25] = a54;
    v[26] = a44;
    v[27] = a34;
    v[28] = a24;
    v[29] = a14;
    v[30] = a5;
    v[31] = a55;
    v[32] = a45;
    v[33] = a35;
    v[34] = a25;
    v[35] = a15;
    v[36] = a2;
    v[37] = a52;
    v[38] = a42;
    v[39] = a32;
    v[40] = a22;
    v[41] = a12;
    v[42] = a1;
    v[43] = a51;
    v[44] = a41;
    v[45] = a31;
    v[46] = a21;
    v[47] = a11;
    v[48] = a8;
    v[49] = a58;
    v[50] = a48;
    v[51] = a38;
    v[52] = a28;
    v[53] = a18;
    v[54] = a9;
    v[55] = a59;
    v[56] = a49;
    v[57] = a39;
    v[58] = a29;
    v[59] = a19;
}

static void o_ntt_64(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33], a34 = v[34], a35 = v[35], a36 = v[36], a37 = v[37], a38 = v[38], a39 = v[39], a40 = v[40], a41 = v[41], a42 = v[42], a43 = v[43], a44 = v[44], a45 = v[45], a46 = v[46], a47 = v[47], a48 = v[48], a49 = v[49], a50 = v[50], a51 = v[51], a52 = v[52], a53 = v[53], a54 = v[54], a55 = v[55], a56 = v[56], a57 = v[57], a58 = v[58], a59 = v[59], a60 = v[60], a61 = v[61], a62 = v[62], a63 = v[63];
    { uint64_t t1 = a0; a0 = o_add(t1, a32); a32 = o_sub(t1, a32); }
    { uint64_t t2 = a8; a8 = o_add(t2, a40); a40 = o_sub(t2, a40); }
    { uint64_t t3 = a16; a16 = o_add(t3, a48); a48 = o_sub(t3, a48); }
    { uint64_t t4 = a24; a24 = o_add(t4, a56); a56 = o_sub(t4, a56); }
    a40 = o_shift(a40, 24);
    a48 = o_shift(a48, 48);
    a56 = o_shift(a56, 72);
    { uint64_t t5 = a0; a0 = o_add(t5, a16); a16 = o_sub(t5, a16); }
    { uint64_t t6 = a8; a8 = o_add(t6, a24); a24 = o_sub(t6, a24); }
    a24 = o_shift(a24, 48);
    { uint64_t t7 = a0; a0 = o_add(t7, a8); a8 = o_sub(t7, a8); }
    { uint64_t t8 = a16; a16 = o_add(t8, a24); a24 = o_sub(t8, a24); }
    { uint64_t t9 = a32; a32 = o_add(t9, a48); a48 = o_sub(t9, a48); }
    { uint64_t t10 = a40; a40 = o_add(t10, a56); a56 = o_sub(t10, a56); }
    a56 = o_shift(a56, 48);
    { uint64_t t11 = a32; a32 = o_add(t11, a40); a40 = o_sub(t11, a40); }
    { uint64_t t12 = a48; a48 = o_add(t12, a56); a56 = o_sub(t12, a56); }
    { uint64_t t13 = a1; a1 = o_add(t13, a33); a33 = o_sub(t13, a33); }
    { uint64_t t14 = a9; a9 = o_add(t14, a41); a41 = o_sub(t14, a41); }
    { uint64_t t15 = a17; a17 = o_add(t15, a49); a49 = o_sub(t15, a49); }
    { uint64_t t16 = a25; a25 = o_add(t16, a57); a57 = o_sub(t16, a57); }
    a41 = o_shift(a41, 24);
    a49 = o_shift(a49, 48);
    a57 = o_shift(a57, 72);
    { uint64_t t17 = a1; a1 = o_add(t17, a17); a17 = o_sub(t17, a17); }
    { uint64_t t18 = a9; a9 = o_add(t18, a25); a25 = o_sub(t18, a25); }
    a25 = o_shift(a25, 48);
    { uint64_t t19 = a1; a1 = o_add(t19, a9); a9 = o_sub(t19, a9); }
    { uint64_t t20 = a17; a17 = o_add(t20, a25); a25 = o_sub(t20, a25); }
    { uint64_t t21 = a33; a33 = o_add(t21, a49); a49 = o_sub(t21, a49); }
    { uint64_t t22 = a41; a41 = o_add(t22, a57); a57 = o_sub(t22, a57); }
    a57 = o_shift(a57, 48);
    { uint64_t t23 = a33; a33 = o_add(t23, a41); a41 = o_sub(t23, a41); }
    { uint64_t t24 = a49; a49 = o_add(t24, a57); a57 = o_sub(t24, a57); }
    { uint64_t t25 = a2; a2 = o_add(t25, a34); a34 = o_sub(t25, a34); }
    { uint64_t t26 = a10; a10 = o_add(t26, a42); a42 = o_sub(t26, a42); }
    { uint64_t t27 = a18; a18 = o_add(t27, a50); a50 = o_sub(t27, a50); }
    { uint64_t t28 = a26; a26 = o_add(t28, a58); a58 = o_sub(t28, a58); }
    a42 = o_shift(a42, 24);
    a50 = o_shift(a50, 48);
    a58 = o_shift(a58, 72);
    { uint64_t t29 = a2; a2 = o_add(t29, a18); a18 = o_sub(t29, a18); }
    { uint64_t t30 = a10; a10 = o_add(t30, a26); a26 = o_sub(t30, a26); }
    a26 = o_shift(a26, 48);
    { uint64_t t31 = a2; a2 = o_add(t31, a10); a10 = o_sub(t31, a10); }
    { uint64_t t32 = a18; a18 = o_add(t32, a26); a26 = o_sub(t32, a26); }
    { uint64_t t33 = a34; a34 = o_add(t33, a50); a50 = o_sub(t33, a50); }
    { uint64_t t34 = a42; a42 = o_add(t34, a58); a58 = o_sub(t34, a58); }
    a58 = o_shift(a58, 48);
    { uint64_t t35 = a34; a34 = o_add(t35, a42); a42 = o_sub(t35, a42); }
    { uint64_t t36 = a50; a50 = o_add(t36, a58); a58 = o_sub(t36, a58); }
    { uint64_t t37 = a3; a3 = o_add(t37, a35); a35 = o_sub(t37, a35); }
    { uint64_t t38 = a11; a11 = o_add(t38, a43); a43 = o_sub(t38, a43); }
    { uint64_t t39 = a19; a19 = o_add(t39, a51); a51 = o_sub(t39, a51); }
    { uint64_t t40 = a27; a27 = o_add(t40, a59); a59 = o_sub(t40, a59); }
    a43 = o_shift(a43, 24);
    a51 = o_shift(a51, 48);
    a59 = o_shift(a59, 72);
    { uint64_t t41 = a3; a3 = o_add(t41, a19); a19 = o_sub(t41, a19); }
    { uint64_t t42 = a11; a11 = o_add(t42, a27); a27 = o_sub(t42, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t43 = a3; a3 = o_add(t43, a11); a11 = o_sub(t43, a11); }
    { uint64_t t44 = a19; a19 = o_add(t44, a27); a27 = o_sub(t44, a27); }
    { uint64_t t45 = a35; a35 = o_add(t45, a51); a51 = o_sub(t45, a51); }
    { uint64_t t46 = a43; a43 = o_add(t46, a59); a59 = o_sub(t46, a59); }
    a59 = o_shift(a59, 48);
    { uint64_t t47 = a35; a35 = o_add(t47, a43); a43 = o_sub(t47, a43); }
    { uint64_t t48 = a51; a51 = o_add(t48, a59); a59 = o_sub(t48, a59); }
    { uint64_t t49 = a4; a4 = o_add(t49, a36); a36 = o_sub(t49, a36); }
    { uint64_t t50 = a12; a12 = o_add(t50, a44); a44 = o_sub(t50, a44); }
    { uint64_t t51 = a20; a20 = o_add(t51, a52); a52 = o_sub(t51, a52); }
    { uint64_t t52 = a28; a28 = o_add(t52, a60); a60 = o_sub(t52, a60); }
    a44 = o_shift(a44, 24);
    a52 = o_shift(a52, 48);
    a60 = o_shift(a60, 72);
    { uint64_t t53 = a4; a4 = o_add(t53, a20); a20 = o_sub(t53, a20); }
    { uint64_t t54 = a12; a12 = o_add(t54, a28); a28 = o_sub(t54, a28); }
    a28 = o_shift(a28, 48);
    { uint64_t t55 = a4; a4 = o_add(t55, a12); a12 = o_sub(t55, a12); }
    { uint64_t t56 = a20; a20 = o_add(t56, a28); a28 = o_sub(t56, a28); }
    { uint64_t t57 = a36; a36 = o_add(t57, a52); a52 = o_sub(t57, a52); }
    { uint64_t t58 = a44; a44 = o_add(t58, a60); a60 = o_sub(t58, a60); }
    a60 = o_shift(a60, 48);
    { uint64_t t59 = a36; a36 = o_add(t59, a44); a44 = o_sub(t59, a44); }
    { uint64_t t60 = a52; a52 = o_add(t60, a60); a60 = o_sub(t60, a60); }
    { uint64_t t61 = a5; a5 = o_add(t61, a37); a37 = o_sub(t61, a37); }
    { uint64_t t62 = a13; a13 = o_add(t62, a45); a45 = o_sub(t62, a45); }
    { uint64_t t63 = a21; a21 = o_add(t63, a53); a53 = o_sub(t63, a53); }
    { uint64_t t64 = a29; a29 = o_add(t64, a61); a61 = o_sub(t64, a61); }
    a45 = o_shift(a45, 24);
    a53 = o_shift(a53, 48);
    a61 = o_shift(a61, 72);
    { uint64_t t65 = a5; a5 = o_add(t65, a21); a21 = o_sub(t65, a21); }
    { uint64_t t66 = a13; a13 = o_add(t66, a29); a29 = o_sub(t66, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t67 = a5; a5 = o_add(t67, a13); a13 = o_sub(t67, a13); }
    { uint64_t t68 = a21; a21 = o_add(t68, a29); a29 = o_sub(t68, a29); }
    { uint64_t t69 = a37; a37 = o_add(t69, a53); a53 = o_sub(t69, a53); }
    { uint64_t t70 = a45; a45 = o_add(t70, a61); a61 = o_sub(t70, a61); }
    a61 = o_shift(a61, 48);
    { uint64_t t71 = a37; a37 = o_add(t71, a45); a45 = o_sub(t71, a45); }
    { uint64_t t72 = a53; a53 = o_add(t72, a61); a61 = o_sub(t72, a61); }
    { uint64_t t73 = a6; a6 = o_add(t73, a38); a38 = o_sub(t73, a38); }
    { uint64_t t74 = a14; a14 = o_add(t74, a46); a46 = o_sub(t74, a46); }
    { uint64_t t75 = a22; a22 = o_add(t75, a54); a54 = o_sub(t75, a54); }
    { uint64_t t76 = a30; a30 = o_add(t76, a62); a62 = o_sub(t76, a62); }
    a46 = o_shift(a46, 24);
    a54 = o_shift(a54, 48);
    a62 = o_shift(a62, 72);
    { uint64_t t77 = a6; a6 = o_add(t77, a22); a22 = o_sub(t77, a22); }
    { uint64_t t78 = a14; a14 = o_add(t78, a30); a30 = o_sub(t78, a30); }
    a30 = o_shift(a30, 48);
    { uint64_t t79 = a6; a6 = o_add(t79, a14); a14 = o_sub(t79, a14); }
    { uint64_t t80 = a22; a22 = o_add(t80, a30); a30 = o_sub(t80, a30); }
    { uint64_t t81 = a38; a38 = o_add(t81, a54); a54 = o_sub(t81, a54); }
    { uint64_t t82 = a46; a46 = o_add(t82, a62); a62 = o_sub(t82, a62); }
    a62 = o_shift(a62, 48);
    { uint64_t t83 = a38; a38 = o_add(t83, a46); a46 = o_sub(t83, a46); }
    { uint64_t t84 = a54; a54 = o_add(t84, a62); a62 = o_sub(t84, a62); }
    { uint64_t t85 = a7; a7 = o_add(t85, a39); a39 = o_sub(t85, a39); }
    { uint64_t t86 = a15; a15 = o_add(t86, a47); a47 = o_sub(t86, a47); }
    { uint64_t t87 = a23; a23 = o_add(t87, a55); a55 = o_sub(t87, a55); }
    { uint64_t t88 = a31; a31 = o_add(t88, a63); a63 = o_sub(t88, a63); }
    a47 = o_shift(a47, 24);
    a55 = o_shift(a55, 48);
    a63 = o_shift(a63, 72);
    { uint64_t t89 = a7; a7 = o_add(t89, a23); a23 = o_sub(t89, a23); }
    { uint64_t t90 = a15; a15 = o_add(t90, a31); a31 = o_sub(t90, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t91 = a7; a7 = o_add(t91, a15); a15 = o_sub(t91, a15); }
    { uint64_t t92 = a23; a23 = o_add(t92, a31); a31 = o_sub(t92, a31); }
    { uint64_t t93 = a39; a39 = o_add(t93, a55); a55 = o_sub(t93, a55); }
    { uint64_t t94 = a47; a47 = o_add(t94, a63); a63 = o_sub(t94, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t95 = a39; a39 = o_add(t95, a47); a47 = o_sub(t95, a47); }
    { uint64_t t96 = a55; a55 = o_add(t96, a63); a63 = o_sub(t96, a63); }
    a33 = o_shift(a33, 3);
    a17 = o_shift(a17, 6);
    a49 = o_shift(a49, 9);
    a9 = o_shift(a9, 12);
    a41 = o_shift(a41, 15);
    a25 = o_shift(a25, 18);
    a57 = o_shift(a57, 21);
    a34 = o_shift(a34, 6);
    a18 = o_shift(a18, 12);
    a50 = o_shift(a50, 18);
    a10 = o_shift(a10, 24);
    a42 = o_shift(a42, 30);
    a26 = o_shift(a26, 36);
    a58 = o_shift(a58, 42);
    a35 = o_shift(a35, 9);
    a19 = o_shift(a19, 18);
    a51 = o_shift(a51, 27);
    a11 = o_shift(a11, 36);
    a43 = o_shift(a43, 45);
    a27 = o_shift(a27, 54);
    a59 = o_shift(a59, 63);
    a36 = o_shift(a36, 12);
    a20 = o_shift(a20, 24);
    a52 = o_shift(a52, 36);
    a12 = o_shift(a12, 48);
    a44 = o_shift(a44, 60);
    a28 = o_shift(a28, 72);
    a60 = o_shift(a60, 84);
    a37 = o_shift(a37, 15);
    a21 = o_shift(a21, 30);
    a53 = o_shift(a53, 45);
    a13 = o_shift(a13, 60);
    a45 = o_shift(a45, 75);
    a29 = o_shift(a29, 90);
    a61 = o_neg(o_shift(a61, 9));
    a38 = o_shift(a38, 18);
    a22 = o_shift(a22, 36);
    a54 = o_shift(a54, 54);
    a14 = o_shift(a14, 72);
    a46 = o_shift(a46, 90);
    a30 = o_neg(o_shift(a30, 12));
    a62 = o_neg(o_shift(a62, 30));
    a39 = o_shift(a39, 21);
    a23 = o_shift(a23, 42);
    a55 = o_shift(a55, 63);
    a15 = o_shift(a15, 84);
    a47 = o_neg(o_shift(a47, 9));
    a31 = o_neg(o_shift(a31, 30));
    a63 = o_neg(o_shift(a63, 51));
    { uint64_t t97 = a0; a0 = o_add(t97, a4); a4 = o_sub(t97, a4); }
    { uint64_t t98 = a1; a1 = o_add(t98, a5); a5 = o_sub(t98, a5); }
    { uint64_t t99 = a2; a2 = o_add(t99, a6); a6 = o_sub(t99, a6); }
    { uint64_t t100 = a3; a3 = o_add(t100, a7); a7 = o_sub(t100, a7); }
    a5 = o_shift(a5, 24);
    a6 = o_shift(a6, 48);
    a7 = o_shift(a7, 72);
    { uint64_t t101 = a0; a0 = o_add(t101, a2); a2 = o_sub(t101, a2); }
    { uint64_t t102 = a1; a1 = o_add(t102, a3); a3 = o_sub(t102, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t103 = a0; a0 = o_add(t103, a1); a1 = o_sub(t103, a1); }
    { uint64_t t104 = a2; a2 = o_add(t104, a3); a3 = o_sub(t104, a3); }
    { uint64_t t105 = a4; a4 = o_add(t105, a6); a6 = o_sub(t105, a6); }
    { uint64_t t106 = a5; a5 = o_add(t106, a7); a7 = o_sub(t106, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t107 = a4; a4 = o_add(t107, a5); a5 = o_sub(t107, a5); }
    { uint64_t t108 = a6; a6 = o_add(t108, a7); a7 = o_sub(t108, a7); }
    { uint64_t t109 = a32; a32 = o_add(t109, a36); a36 = o_sub(t109, a36); }
    { uint64_t t110 = a33; a33 = o_add(t110, a37); a37 = o_sub(t110, a37); }
    { uint64_t t111 = a34; a34 = o_add(t111, a38); a38 = o_sub(t111, a38); }
    { uint64_t t112 = a35; a35 = o_add(t112, a39); a39 = o_sub(t112, a39); }
    a37 = o_shift(a37, 24);
    a38 = o_shift(a38, 48);
    a39 = o_shift(a39, 72);
    { uint64_t t113 = a32; a32 = o_add(t113, a34); a34 = o_sub(t113, a34); }
    { uint64_t t114 = a33; a33 = o_add(t114, a35); a35 = o_sub(t114, a35); }
    a35 = o_shift(a35, 48);
    { uint64_t t115 = a32; a32 = o_add(t115, a33); a33 = o_sub(t115, a33); }
    { uint64_t t116 = a34; a34 = o_add(t116, a35); a35 = o_sub(t116, a35); }
    { uint64_t t117 = a36; a36 = o_add(t117, a38); a38 = o_sub(t117, a38); }
    { uint64_t t118 = a37; a37 = o_add(t118, a39); a39 = o_sub(t118, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t119 = a36; a36 = o_add(t119, a37); a37 = o_sub(t119, a37); }
    { uint64_t t120 = a38; a38 = o_add(t120, a39); a39 = o_sub(t120, a39); }
    { uint64_t t121 = a16; a16 = o_add(t121, a20); a20 = o_sub(t121, a20); }
    { uint64_t t122 = a17; a17 = o_add(t122, a21); a21 = o_sub(t122, a21); }
    { uint64_t t123 = a18; a18 = o_add(t123, a22); a22 = o_sub(t123, a22); }
    { uint64_t t124 = a19; a19 = o_add(t124, a23); a23 = o_sub(t124, a23); }
    a21 = o_shift(a21, 24);
    a22 = o_shift(a22, 48);
    a23 = o_shift(a23, 72);
    { uint64_t t125 = a16; a16 = o_add(t125, a18); a18 = o_sub(t125, a18); }
    { uint64_t t126 = a17; a17 = o_add(t126, a19); a19 = o_sub(t126, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t127 = a16; a16 = o_add(t127, a17); a17 = o_sub(t127, a17); }
    { uint64_t t128 = a18; a18 = o_add(t128, a19); a19 = o_sub(t128, a19); }
    { uint64_t t129 = a20; a20 = o_add(t129, a22); a22 = o_sub(t129, a22); }
    { uint64_t t130 = a21; a21 = o_add(t130, a23); a23 = o_sub(t130, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t131 = a20; a20 = o_add(t131, a21); a21 = o_sub(t131, a21); }
    { uint64_t t132 = a22; a22 = o_add(t132, a23); a23 = o_sub(t132, a23); }
    { uint64_t t133 = a48; a48 = o_add(t133, a52); a52 = o_sub(t133, a52); }
    { uint64_t t134 = a49; a49 = o_add(t134, a53); a53 = o_sub(t134, a53); }
    { uint64_t t135 = a50; a50 = o_add(t135, a54); a54 = o_sub(t135, a54); }
    { uint64_t t136 = a51; a51 = o_add(t136, a55); a55 = o_sub(t136, a55); }
    a53 = o_shift(a53, 24);
    a54 = o_shift(a54, 48);
    a55 = o_shift(a55, 72);
    { uint64_t t137 = a48; a48 = o_add(t137, a50); a50 = o_sub(t137, a50); }
    { uint64_t t138 = a49; a49 = o_add(t138, a51); a51 = o_sub(t138, a51); }
    a51 = o_shift(a51, 48);
    { uint64_t t139 = a48; a48 = o_add(t139, a49); a49 = o_sub(t139, a49); }
    { uint64_t t140 = a50; a50 = o_add(t140, a51); a51 = o_sub(t140, a51); }
    { uint64_t t141 = a52; a52 = o_add(t141, a54); a54 = o_sub(t141, a54); }
    { uint64_t t142 = a53; a53 = o_add(t142, a55); a55 = o_sub(t142, a55); }
    a55 = o_shift(a55, 48);
    { uint64_t t143 = a52; a52 = o_add(t143, a53); a53 = o_sub(t143, a53); }
    { uint64_t t144 = a54; a54 = o_add(t144, a55); a55 = o_sub(t144, a55); }
    { uint64_t t145 = a8; a8 = o_add(t145, a12); a12 = o_sub(t145, a12); }
    { uint64_t t146 = a9; a9 = o_add(t146, a13); a13 = o_sub(t146, a13); }
    { uint64_t t147 = a10; a10 = o_add(t147, a14); a14 = o_sub(t147, a14); }
    { uint64_t t148 = a11; a11 = o_add(t148, a15); a15 = o_sub(t148, a15); }
    a13 = o_shift(a13, 24);
    a14 = o_shift(a14, 48);
    a15 = o_shift(a15, 72);
    { uint64_t t149 = a8; a8 = o_add(t149, a10); a10 = o_sub(t149, a10); }
    { uint64_t t150 = a9; a9 = o_add(t150, a11); a11 = o_sub(t150, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t151 = a8; a8 = o_add(t151, a9); a9 = o_sub(t151, a9); }
    { uint64_t t152 = a10; a10 = o_add(t152, a11); a11 = o_sub(t152, a11); }
    { uint64_t t153 = a12; a12 = o_add(t153, a14); a14 = o_sub(t153, a14); }
    { uint64_t t154 = a13; a13 = o_add(t154, a15); a15 = o_sub(t154, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t155 = a12; a12 = o_add(t155, a13); a13 = o_sub(t155, a13); }
    { uint64_t t156 = a14; a14 = o_add(t156, a15); a15 = o_sub(t156, a15); }
    { uint64_t t157 = a40; a40 = o_add(t157, a44); a44 = o_sub(t157, a44); }
    { uint64_t t158 = a41; a41 = o_add(t158, a45); a45 = o_sub(t158, a45); }
    { uint64_t t159 = a42; a42 = o_add(t159, a46); a46 = o_sub(t159, a46); }
    { uint64_t t160 = a43; a43 = o_add(t160, a47); a47 = o_sub(t160, a47); }
    a45 = o_shift(a45, 24);
    a46 = o_shift(a46, 48);
    a47 = o_shift(a47, 72);
    { uint64_t t161 = a40; a40 = o_add(t161, a42); a42 = o_sub(t161, a42); }
    { uint64_t t162 = a41; a41 = o_add(t162, a43); a43 = o_sub(t162, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t163 = a40; a40 = o_add(t163, a41); a41 = o_sub(t163, a41); }
    { uint64_t t164 = a42; a42 = o_add(t164, a43); a43 = o_sub(t164, a43); }
    { uint64_t t165 = a44; a44 = o_add(t165, a46); a46 = o_sub(t165, a46); }
    { uint64_t t166 = a45; a45 = o_add(t166, a47); a47 = o_sub(t166, a47); }
    a47 = o_shift(a47, 48);
    { uint64_t t167 = a44; a44 = o_add(t167, a45); a45 = o_sub(t167, a45); }
    { uint64_t t168 = a46; a46 = o_add(t168, a47); a47 = o_sub(t168, a47); }
    { uint64_t t169 = a24; a24 = o_add(t169, a28); a28 = o_sub(t169, a28); }
    { uint64_t t170 = a25; a25 = o_add(t170, a29); a29 = o_sub(t170, a29); }
    { uint64_t t171 = a26; a26 = o_add(t171, a30); a30 = o_sub(t171, a30); }
    { uint64_t t172 = a27; a27 = o_add(t172, a31); a31 = o_sub(t172, a31); }
    a29 = o_shift(a29, 24);
    a30 = o_shift(a30, 48);
    a31 = o_shift(a31, 72);
    { uint64_t t173 = a24; a24 = o_add(t173, a26); a26 = o_sub(t173, a26); }
    { uint64_t t174 = a25; a25 = o_add(t174, a27); a27 = o_sub(t174, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t175 = a24; a24 = o_add(t175, a25); a25 = o_sub(t175, a25); }
    { uint64_t t176 = a26; a26 = o_add(t176, a27); a27 = o_sub(t176, a27); }
    { uint64_t t177 = a28; a28 = o_add(t177, a30); a30 = o_sub(t177, a30); }
    { uint64_t t178 = a29; a29 = o_add(t178, a31); a31 = o_sub(t178, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t179 = a28; a28 = o_add(t179, a29); a29 = o_sub(t179, a29); }
    { uint64_t t180 = a30; a30 = o_add(t180, a31); a31 = o_sub(t180, a31); }
    { uint64_t t181 = a56; a56 = o_add(t181, a60); a60 = o_sub(t181, a60); }
    { uint64_t t182 = a57; a57 = o_add(t182, a61); a61 = o_sub(t182, a61); }
    { uint64_t t183 = a58; a58 = o_add(t183, a62); a62 = o_sub(t183, a62); }
    { uint64_t t184 = a59; a59 = o_add(t184, a63); a63 = o_sub(t184, a63); }
    a61 = o_shift(a61, 24);
    a62 = o_shift(a62, 48);
    a63 = o_shift(a63, 72);
    { uint64_t t185 = a56; a56 = o_add(t185, a58); a58 = o_sub(t185, a58); }
    { uint64_t t186 = a57; a57 = o_add(t186, a59); a59 = o_sub(t186, a59); }
    a59 = o_shift(a59, 48);
    { uint64_t t187 = a56; a56 = o_add(t187, a57); a57 = o_sub(t187, a57); }
    { uint64_t t188 = a58; a58 = o_add(t188, a59); a59 = o_sub(t188, a59); }
    { uint64_t t189 = a60; a60 = o_add(t189, a62); a62 = o_sub(t189, a62); }
    { uint64_t t190 = a61; a61 = o_add(t190, a63); a63 = o_sub(t190, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t191 = a60; a60 = o_add(t191, a61); a61 = o_sub(t191, a61); }
    { uint64_t t192 = a62; a62 = o_add(t192, a63); a63 = o_sub(t192, a63); }
    v[0] = a0;
    v[1] = a32;
    v[2] = a16;
    v[3] = a48;
    v[4] = a8;
    v[5] = a40;
    v[6] = a24;
    v[7] = a56;
    v[8] = a4;
    v[9] = a36;
    v[10] = a20;
    v[11] = a52;
    v[12] = a12;
    v[13] = a44;
    v[14] = a28;
    v[15] = a60;
    v[16] = a2;
    v[17] = a34;
    v[18] = a18;
    v[19] = a50;
    v[20] = a10;
    v[21] = a42;
    v[22] = a26;
    v[23] = a58;
    v[24] = a6;
    v[25] = a38;
    v[26] = a22;
    v[27] = a54;
    v[28] = a14;
    v[29] = a46;
    v[30] = a30;
    v[31] = a62;
    v[32] = a1;
    v[33] = a33;
    v[34] = a17;
    v[35] = a49;
    v[36] = a9;
    v[37] = a41;
    v[38] = a25;
    v[39] = a57;
    v[40] = a5;
    v[41] = a37;
    v[42] = a21;
    v[43] = a53;
    v[44] = a13;
    v[45] = a45;
    v[46] = a29;
    v[47] = a61;
    v[48] = a3;
    v[49] = a35;
    v[50] = a19;
    v[51] = a51;
    v[52] = a11;
    v[53] = a43;
    v[54] = a27;
    v[55] = a59;
    v[56] = a7;
    v[57] = a39;
    v[58] = a23;
    v[59] = a55;
    v[60] = a15;
    v[61] = a47;
    v[62] = a31;
    v[63] = a63;
}

static void o_ntt_68(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33], a34 = v[34], a35 = v[35], a36 = v[36], a37 = v[37], a38 = v[38], a39 = v[39], a40 = v[40], a41 = v[41], a42 = v[42], a43 = v[43], a44 = v[44], a45 = v[45], a46 = v[46], a47 = v[47], a48 = v[48], a49 = v[49], a50 = v[50], a51 = v[51], a52 = v[52], a53 = v[53], a54 = v[54], a55 = v[55], a56 = v[56], a57 = v[57], a58 = v[58], a59 = v[59], a60 = v[60], a61 = v[61], a62 = v[62], a63 = v[63], a64 = v[64], a65 = v[65], a66 = v[66], a67 = v[67];
    { uint64_t t1 = a4; a4 = o_add(t1, a64); a64 = o_sub(t1, a64); }
    { uint64_t t2 = a16; a16 = o_add(t2, a52); a52 = o_sub(t2, a52); }
    a52 = o_shift(a52, 48);
    { uint64_t t3 = a4; a4 = o_add(t3, a16); a16 = o_sub(t3, a16); }
    { uint64_t t4 = a64; a64 = o_add(t4, a52); a52 = o_sub(t4, a52); }
    { uint64_t t5 = a24; a24 = o_add(t5, a44); a44 = o_sub(t5, a44); }
    { uint64_t t6 = a28; a28 = o_add(t6, a40); a40 = o_sub(t6, a40); }
    a40 = o_shift(a40, 48);
    { uint64_t t7 = a24; a24 = o_add(t7, a28); a28 = o_sub(t7, a28); }
    { uint64_t t8 = a44; a44 = o_add(t8, a40); a40 = o_sub(t8, a40); }
    { uint64_t t9 = a8; a8 = o_add(t9, a60); a60 = o_sub(t9, a60); }
    { uint64_t t10 = a32; a32 = o_add(t10, a36); a36 = o_sub(t10, a36); }
    a36 = o_shift(a36, 48);
    { uint64_t t11 = a8; a8 = o_add(t11, a32); a32 = o_sub(t11, a32); }
    { uint64_t t12 = a60; a60 = o_add(t12, a36); a36 = o_sub(t12, a36); }
    { uint64_t t13 = a48; a48 = o_add(t13, a20); a20 = o_sub(t13, a20); }
    { uint64_t t14 = a56; a56 = o_add(t14, a12); a12 = o_sub(t14, a12); }
    a12 = o_shift(a12, 48);
    { uint64_t t15 = a48; a48 = o_add(t15, a56); a56 = o_sub(t15, a56); }
    { uint64_t t16 = a20; a20 = o_add(t16, a12); a12 = o_sub(t16, a12); }
    a44 = o_shift(a44, 12);
    a28 = o_shift(a28, 24);
    a40 = o_shift(a40, 36);
    a60 = o_shift(a60, 24);
    a32 = o_shift(a32, 48);
    a36 = o_shift(a36, 72);
    a20 = o_shift(a20, 36);
    a56 = o_shift(a56, 72);
    a12 = o_neg(o_shift(a12, 12));
    { uint64_t t17 = a4; a4 = o_add(t17, a8); a8 = o_sub(t17, a8); }
    { uint64_t t18 = a24; a24 = o_add(t18, a48); a48 = o_sub(t18, a48); }
    a48 = o_shift(a48, 48);
    { uint64_t t19 = a4; a4 = o_add(t19, a24); a24 = o_sub(t19, a24); }
    { uint64_t t20 = a8; a8 = o_add(t20, a48); a48 = o_sub(t20, a48); }
    { uint64_t t21 = a64; a64 = o_add(t21, a60); a60 = o_sub(t21, a60); }
    { uint64_t t22 = a44; a44 = o_add(t22, a20); a20 = o_sub(t22, a20); }
    a20 = o_shift(a20, 48);
    { uint64_t t23 = a64; a64 = o_add(t23, a44); a44 = o_sub(t23, a44); }
    { uint64_t t24 = a60; a60 = o_add(t24, a20); a20 = o_sub(t24, a20); }
    { uint64_t t25 = a16; a16 = o_add(t25, a32); a32 = o_sub(t25, a32); }
    { uint64_t t26 = a28; a28 = o_add(t26, a56); a56 = o_sub(t26, a56); }
    a56 = o_shift(a56, 48);
    { uint64_t t27 = a16; a16 = o_add(t27, a28); a28 = o_sub(t27, a28); }
    { uint64_t t28 = a32; a32 = o_add(t28, a56); a56 = o_sub(t28, a56); }
    { uint64_t t29 = a52; a52 = o_add(t29, a36); a36 = o_sub(t29, a36); }
    { uint64_t t30 = a40; a40 = o_add(t30, a12); a12 = o_sub(t30, a12); }
    a12 = o_shift(a12, 48);
    { uint64_t t31 = a52; a52 = o_add(t31, a40); a40 = o_sub(t31, a40); }
    { uint64_t t32 = a36; a36 = o_add(t32, a12); a12 = o_sub(t32, a12); }
    uint64_t t33 = a0;
    a0 = o_add(a0, a4);
    a4 = o_mul(a4, 1152921504338411520ULL);
    a64 = o_mul(a64, 6259776822214049175ULL);
    a16 = o_mul(a16, 9380094172986290191ULL);
    a52 = o_mul(a52, 891943630314919127ULL);
    a8 = o_mul(a8, 17228171707553225791ULL);
    a60 = o_mul(a60, 12855743360534130886ULL);
    a32 = o_mul(a32, 6167687396920564837ULL);
    a36 = o_mul(a36, 17201834061724655524ULL);
    a24 = o_mul(a24, 15308299771656910737ULL);
    a44 = o_mul(a44, 18186005861103657533ULL);
    a28 = o_mul(a28, 53595491891823545ULL);
    a40 = o_mul(a40, 1906638201581172103ULL);
    a48 = o_mul(a48, 18303651001328874822ULL);
    a20 = o_mul(a20, 3077466521755967626ULL);
    a56 = o_mul(a56, 12423593102987598328ULL);
    a12 = o_mul(a12, 18361513053649472048ULL);
    a4 = o_add(a4, t33);
    { uint64_t t34 = a4; a4 = o_add(t34, a24); a24 = o_sub(t34, a24); }
    { uint64_t t35 = a48; a48 = o_add(t35, a8); a8 = o_sub(t35, a8); }
    a8 = o_shift(a8, 48);
    { uint64_t t36 = a4; a4 = o_add(t36, a48); a48 = o_sub(t36, a48); }
    { uint64_t t37 = a24; a24 = o_add(t37, a8); a8 = o_sub(t37, a8); }
    { uint64_t t38 = a12; a12 = o_add(t38, a36); a36 = o_sub(t38, a36); }
    { uint64_t t39 = a40; a40 = o_add(t39, a52); a52 = o_sub(t39, a52); }
    a52 = o_shift(a52, 48);
    { uint64_t t40 = a12; a12 = o_add(t40, a40); a40 = o_sub(t40, a40); }
    { uint64_t t41 = a36; a36 = o_add(t41, a52); a52 = o_sub(t41, a52); }
    { uint64_t t42 = a56; a56 = o_add(t42, a32); a32 = o_sub(t42, a32); }
    { uint64_t t43 = a28; a28 = o_add(t43, a16); a16 = o_sub(t43, a16); }
    a16 = o_shift(a16, 48);
    { uint64_t t44 = a56; a56 = o_add(t44, a28); a28 = o_sub(t44, a28); }
    { uint64_t t45 = a32; a32 = o_add(t45, a16); a16 = o_sub(t45, a16); }
    { uint64_t t46 = a20; a20 = o_add(t46, a60); a60 = o_sub(t46, a60); }
    { uint64_t t47 = a44; a44 = o_add(t47, a64); a64 = o_sub(t47, a64); }
    a64 = o_shift(a64, 48);
    { uint64_t t48 = a20; a20 = o_add(t48, a44); a44 = o_sub(t48, a44); }
    { uint64_t t49 = a60; a60 = o_add(t49, a64); a64 = o_sub(t49, a64); }
    a36 = o_shift(a36, 12);
    a40 = o_shift(a40, 24);
    a52 = o_shift(a52, 36);
    a32 = o_shift(a32, 24);
    a28 = o_shift(a28, 48);
    a16 = o_shift(a16, 72);
    a60 = o_shift(a60, 36);
    a44 = o_shift(a44, 72);
    a64 = o_neg(o_shift(a64, 12));
    { uint64_t t50 = a4; a4 = o_add(t50, a56); a56 = o_sub(t50, a56); }
    { uint64_t t51 = a12; a12 = o_add(t51, a20); a20 = o_sub(t51, a20); }
    a20 = o_shift(a20, 48);
    { uint64_t t52 = a4; a4 = o_add(t52, a12); a12 = o_sub(t52, a12); }
    { uint64_t t53 = a56; a56 = o_add(t53, a20); a20 = o_sub(t53, a20); }
    { uint64_t t54 = a24; a24 = o_add(t54, a32); a32 = o_sub(t54, a32); }
    { uint64_t t55 = a36; a36 = o_add(t55, a60); a60 = o_sub(t55, a60); }
    a60 = o_shift(a60, 48);
    { uint64_t t56 = a24; a24 = o_add(t56, a36); a36 = o_sub(t56, a36); }
    { uint64_t t57 = a32; a32 = o_add(t57, a60); a60 = o_sub(t57, a60); }
    { uint64_t t58 = a48; a48 = o_add(t58, a28); a28 = o_sub(t58, a28); }
    { uint64_t t59 = a40; a40 = o_add(t59, a44); a44 = o_sub(t59, a44); }
    a44 = o_shift(a44, 48);
    { uint64_t t60 = a48; a48 = o_add(t60, a40); a40 = o_sub(t60, a40); }
    { uint64_t t61 = a28; a28 = o_add(t61, a44); a44 = o_sub(t61, a44); }
    { uint64_t t62 = a8; a8 = o_add(t62, a16); a16 = o_sub(t62, a16); }
    { uint64_t t63 = a52; a52 = o_add(t63, a64); a64 = o_sub(t63, a64); }
    a64 = o_shift(a64, 48);
    { uint64_t t64 = a8; a8 = o_add(t64, a52); a52 = o_sub(t64, a52); }
    { uint64_t t65 = a16; a16 = o_add(t65, a64); a64 = o_sub(t65, a64); }
    { uint64_t t66 = a21; a21 = o_add(t66, a13); a13 = o_sub(t66, a13); }
    { uint64_t t67 = a33; a33 = o_add(t67, a1); a1 = o_sub(t67, a1); }
    a1 = o_shift(a1, 48);
    { uint64_t t68 = a21; a21 = o_add(t68, a33); a33 = o_sub(t68, a33); }
    { uint64_t t69 = a13; a13 = o_add(t69, a1); a1 = o_sub(t69, a1); }
    { uint64_t t70 = a41; a41 = o_add(t70, a61); a61 = o_sub(t70, a61); }
    { uint64_t t71 = a45; a45 = o_add(t71, a57); a57 = o_sub(t71, a57); }
    a57 = o_shift(a57, 48);
    { uint64_t t72 = a41; a41 = o_add(t72, a45); a45 = o_sub(t72, a45); }
    { uint64_t t73 = a61; a61 = o_add(t73, a57); a57 = o_sub(t73, a57); }
    { uint64_t t74 = a25; a25 = o_add(t74, a9); a9 = o_sub(t74, a9); }
    { uint64_t t75 = a49; a49 = o_add(t75, a53); a53 = o_sub(t75, a53); }
    a53 = o_shift(a53, 48);
    { uint64_t t76 = a25; a25 = o_add(t76, a49); a49 = o_sub(t76, a49); }
    { uint64_t t77 = a9; a9 = o_add(t77, a53); a53 = o_sub(t77, a53); }
    { uint64_t t78 = a65; a65 = o_add(t78, a37); a37 = o_sub(t78, a37); }
    { uint64_t t79 = a5; a5 = o_add(t79, a29); a29 = o_sub(t79, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t80 = a65; a65 = o_add(t80, a5); a5 = o_sub(t80, a5); }
    { uint64_t t81 = a37; a37 = o_add(t81, a29); a29 = o_sub(t81, a29); }
    a61 = o_shift(a61, 12);
    a45 = o_shift(a45, 24);
    a57 = o_shift(a57, 36);
    a9 = o_shift(a9, 24);
    a49 = o_shift(a49, 48);
    a53 = o_shift(a53, 72);
    a37 = o_shift(a37, 36);
    a5 = o_shift(a5, 72);
    a29 = o_neg(o_shift(a29, 12));
    { uint64_t t82 = a21; a21 = o_add(t82, a25); a25 = o_sub(t82, a25); }
    { uint64_t t83 = a41; a41 = o_add(t83, a65); a65 = o_sub(t83, a65); }
    a65 = o_shift(a65, 48);
    { uint64_t t84 = a21; a21 = o_add(t84, a41); a41 = o_sub(t84, a41); }
    { uint64_t t85 = a25; a25 = o_add(t85, a65); a65 = o_sub(t85, a65); }
    { uint64_t t86 = a13; a13 = o_add(t86, a9); a9 = o_sub(t86, a9); }
    { uint64_t t87 = a61; a61 = o_add(t87, a37); a37 = o_sub(t87, a37); }
    a37 = o_shift(a37, 48);
    { uint64_t t88 = a13; a13 = o_add(t88, a61); a61 = o_sub(t88, a61); }
    { uint64_t t89 = a9; a9 = o_add(t89, a37); a37 = o_sub(t89, a37); }
    { uint64_t t90 = a33; a33 = o_add(t90, a49); a49 = o_sub(t90, a49); }
    { uint64_t t91 = a45; a45 = o_add(t91, a5); a5 = o_sub(t91, a5); }
    a5 = o_shift(a5, 48);
    { uint64_t t92 = a33; a33 = o_add(t92, a45); a45 = o_sub(t92, a45); }
    { uint64_t t93 = a49; a49 = o_add(t93, a5); a5 = o_sub(t93, a5); }
    { uint64_t t94 = a1; a1 = o_add(t94, a53); a53 = o_sub(t94, a53); }
    { uint64_t t95 = a57; a57 = o_add(t95, a29); a29 = o_sub(t95, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t96 = a1; a1 = o_add(t96, a57); a57 = o_sub(t96, a57); }
    { uint64_t t97 = a53; a53 = o_add(t97, a29); a29 = o_sub(t97, a29); }
    uint64_t t98 = a17;
    a17 = o_add(a17, a21);
    a21 = o_mul(a21, 1152921504338411520ULL);
    a13 = o_mul(a13, 6259776822214049175ULL);
    a33 = o_mul(a33, 9380094172986290191ULL);
    a1 = o_mul(a1, 891943630314919127ULL);
    a25 = o_mul(a25, 17228171707553225791ULL);
    a9 = o_mul(a9, 12855743360534130886ULL);
    a49 = o_mul(a49, 6167687396920564837ULL);
    a53 = o_mul(a53, 17201834061724655524ULL);
    a41 = o_mul(a41, 15308299771656910737ULL);
    a61 = o_mul(a61, 18186005861103657533ULL);
    a45 = o_mul(a45, 53595491891823545ULL);
    a57 = o_mul(a57, 1906638201581172103ULL);
    a65 = o_mul(a65, 18303651001328874822ULL);
    a37 = o_mul(a37, 3077466521755967626ULL);
    a5 = o_mul(a5, 12423593102987598328ULL);
    a29 = o_mul(a29, 18361513053649472048ULL);
    a21 = o_add(a21, t98);
    { uint64_t t99 = a21; a21 = o_add(t99, a41); a41 = o_sub(t99, a41); }
    { uint64_t t100 = a65; a65 = o_add(t100, a25); a25 = o_sub(t100, a25); }
    a25 = o_shift(a25, 48);
    { uint64_t t101 = a21; a21 = o_add(t101, a65); a65 = o_sub(t101, a65); }
    { uint64_t t102 = a41; a41 = o_add(t102, a25); a25 = o_sub(t102, a25); }
    { uint64_t t103 = a29; a29 = o_add(t103, a53); a53 = o_sub(t103, a53); }
    { uint64_t t104 = a57; a57 = o_add(t104, a1); a1 = o_sub(t104, a1); }
    a1 = o_shift(a1, 48);
    { uint64_t t105 = a29; a29 = o_add(t105, a57); a57 = o_sub(t105, a57); }
    { uint64_t t106 = a53; a53 = o_add(t106, a1); a1 = o_sub(t106, a1); }
    { uint64_t t107 = a5; a5 = o_add(t107, a49); a49 = o_sub(t107, a49); }
    { uint64_t t108 = a45; a45 = o_add(t108, a33); a33 = o_sub(t108, a33); }
    a33 = o_shift(a33, 48);
    { uint64_t t109 = a5; a5 = o_add(t109, a45); a45 = o_sub(t109, a45); }
    { uint64_t t110 = a49; a49 = o_add(t110, a33); a33 = o_sub(t110, a33); }
    { uint64_t t111 = a37; a37 = o_add(t111, a9); a9 = o_sub(t111, a9); }
    { uint64_t t112 = a61; a61 = o_add(t112, a13); a13 = o_sub(t112, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t113 = a37; a37 = o_add(t113, a61); a61 = o_sub(t113, a61); }
    { uint64_t t114 = a9; a9 = o_add(t114, a13); a13 = o_sub(t114, a13); }
    a53 = o_shift(a53, 12);
    a57 = o_shift(a57, 24);
    a1 = o_shift(a1, 36);
    a49 = o_shift(a49, 24);
    a45 = o_shift(a45, 48);
    a33 = o_shift(a33, 72);
    a9 = o_shift(a9, 36);
    a61 = o_shift(a61, 72);
    a13 = o_neg(o_shift(a13, 12));
    { uint64_t t115 = a21; a21 = o_add(t115, a5); a5 = o_sub(t115, a5); }
    { uint64_t t116 = a29; a29 = o_add(t116, a37); a37 = o_sub(t116, a37); }
    a37 = o_shift(a37, 48);
    { uint64_t t117 = a21; a21 = o_add(t117, a29); a29 = o_sub(t117, a29); }
    { uint64_t t118 = a5; a5 = o_add(t118, a37); a37 = o_sub(t118, a37); }
    { uint64_t t119 = a41; a41 = o_add(t119, a49); a49 = o_sub(t119, a49); }
    { uint64_t t120 = a53; a53 = o_add(t120, a9); a9 = o_sub(t120, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t121 = a41; a41 = o_add(t121, a53); a53 = o_sub(t121, a53); }
    { uint64_t t122 = a49; a49 = o_add(t122, a9); a9 = o_sub(t122, a9); }
    { uint64_t t123 = a65; a65 = o_add(t123, a45); a45 = o_sub(t123, a45); }
    { uint64_t t124 = a57; a57 = o_add(t124, a61); a61 = o_sub(t124, a61); }
    a61 = o_shift(a61, 48);
    { uint64_t t125 = a65; a65 = o_add(t125, a57); a57 = o_sub(t125, a57); }
    { uint64_t t126 = a45; a45 = o_add(t126, a61); a61 = o_sub(t126, a61); }
    { uint64_t t127 = a25; a25 = o_add(t127, a33); a33 = o_sub(t127, a33); }
    { uint64_t t128 = a1; a1 = o_add(t128, a13); a13 = o_sub(t128, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t129 = a25; a25 = o_add(t129, a1); a1 = o_sub(t129, a1); }
    { uint64_t t130 = a33; a33 = o_add(t130, a13); a13 = o_sub(t130, a13); }
    { uint64_t t131 = a38; a38 = o_add(t131, a30); a30 = o_sub(t131, a30); }
    { uint64_t t132 = a50; a50 = o_add(t132, a18); a18 = o_sub(t132, a18); }
    a18 = o_shift(a18, 48);
    { uint64_t t133 = a38; a38 = o_add(t133, a50); a50 = o_sub(t133, a50); }
    { uint64_t t134 = a30; a30 = o_add(t134, a18); a18 = o_sub(t134, a18); }
    { uint64_t t135 = a58; a58 = o_add(t135, a10); a10 = o_sub(t135, a10); }
    { uint64_t t136 = a62; a62 = o_add(t136, a6); a6 = o_sub(t136, a6); }
    a6 = o_shift(a6, 48);
    { uint64_t t137 = a58; a58 = o_add(t137, a62); a62 = o_sub(t137, a62); }
    { uint64_t t138 = a10; a10 = o_add(t138, a6); a6 = o_sub(t138, a6); }
    { uint64_t t139 = a42; a42 = o_add(t139, a26); a26 = o_sub(t139, a26); }
    { uint64_t t140 = a66; a66 = o_add(t140, a2); a2 = o_sub(t140, a2); }
    a2 = o_shift(a2, 48);
    { uint64_t t141 = a42; a42 = o_add(t141, a66); a66 = o_sub(t141, a66); }
    { uint64_t t142 = a26; a26 = o_add(t142, a2); a2 = o_sub(t142, a2); }
    { uint64_t t143 = a14; a14 = o_add(t143, a54); a54 = o_sub(t143, a54); }
    { uint64_t t144 = a22; a22 = o_add(t144, a46); a46 = o_sub(t144, a46); }
    a46 = o_shift(a46, 48);
    { uint64_t t145 = a14; a14 = o_add(t145, a22); a22 = o_sub(t145, a22); }
    { uint64_t t146 = a54; a54 = o_add(t146, a46); a46 = o_sub(t146, a46); }
    a10 = o_shift(a10, 12);
    a62 = o_shift(a62, 24);
    a6 = o_shift(a6, 36);
    a26 = o_shift(a26, 24);
    a66 = o_shift(a66, 48);
    a2 = o_shift(a2, 72);
    a54 = o_shift(a54, 36);
    a22 = o_shift(a22, 72);
    a46 = o_neg(o_shift(a46, 12));
    { uint64_t t147 = a38; a38 = o_add(t147, a42); a42 = o_sub(t147, a42); }
    { uint64_t t148 = a58; a58 = o_add(t148, a14); a14 = o_sub(t148, a14); }
    a14 = o_shift(a14, 48);
    { uint64_t t149 = a38; a38 = o_add(t149, a58); a58 = o_sub(t149, a58); }
    { uint64_t t150 = a42; a42 = o_add(t150, a14); a14 = o_sub(t150, a14); }
    { uint64_t t151 = a30; a30 = o_add(t151, a26); a26 = o_sub(t151, a26); }
    { uint64_t t152 = a10; a10 = o_add(t152, a54); a54 = o_sub(t152, a54); }
    a54 = o_shift(a54, 48);
    { uint64_t t153 = a30; a30 = o_add(t153, a10); a10 = o_sub(t153, a10); }
    { uint64_t t154 = a26; a26 = o_add(t154, a54); a54 = o_sub(t154, a54); }
    { uint64_t t155 = a50; a50 = o_add(t155, a66); a66 = o_sub(t155, a66); }
    { uint64_t t156 = a62; a62 = o_add(t156, a22); a22 = o_sub(t156, a22); }
    a22 = o_shift(a22, 48);
    { uint64_t t157 = a50; a50 = o_add(t157, a62); a62 = o_sub(t157, a62); }
    { uint64_t t158 = a66; a66 = o_add(t158, a22); a22 = o_sub(t158, a22); }
    { uint64_t t159 = a18; a18 = o_add(t159, a2); a2 = o_sub(t159, a2); }
    { uint64_t t160 = a6; a6 = o_add(t160, a46); a46 = o_sub(t160, a46); }
    a46 = o_shift(a46, 48);
    { uint64_t t161 = a18; a18 = o_add(t161, a6); a6 = o_sub(t161, a6); }
    { uint64_t t162 = a2; a2 = o_add(t162, a46); a46 = o_sub(t162, a46); }
    uint64_t t163 = a34;
    a34 = o_add(a34, a38);
    a38 = o_mul(a38, 1152921504338411520ULL);
    a30 = o_mul(a30, 6259776822214049175ULL);
    a50 = o_mul(a50, 9380094172986290191ULL);
    a18 = o_mul(a18, 891943630314919127ULL);
    a42 = o_mul(a42, 17228171707553225791ULL);
    a26 = o_mul(a26, 12855743360534130886ULL);
    a66 = o_mul(a66, 6167687396920564837ULL);
    a2 = o_mul(a2, 17201834061724655524ULL);
    a58 = o_mul(a58, 15308299771656910737ULL);
    a10 = o_mul(a10, 18186005861103657533ULL);
    a62 = o_mul(a62, 53595491891823545ULL);
    a6 = o_mul(a6, 1906638201581172103ULL);
    a14 = o_mul(a14, 18303651001328874822ULL);
    a54 = o_mul(a54, 3077466521755967626ULL);
    a22 = o_mul(a22, 12423593102987598328ULL);
    a46 = o_mul(a46, 18361513053649472048ULL);
    a38 = o_add(a38, t163);
    { uint64_t t164 = a38; a38 = o_add(t164, a58); a58 = o_sub(t164, a58); }
    { uint64_t t165 = a14; a14 = o_add(t165, a42); a42 = o_sub(t165, a42); }
    a42 = o_shift(a42, 48);
    { uint64_t t166 = a38; a38 = o_add(t166, a14); a14 = o_sub(t166, a14); }
    { uint64_t t167 = a58; a58 = o_add(t167, a42); a42 = o_sub(t167, a42); }
    { uint64_t t168 = a46; a46 = o_add(t168, a2); a2 = o_sub(t168, a2); }
    { uint64_t t169 = a6; a6 = o_add(t169, a18); a18 = o_sub(t169, a18); }
    a18 = o_shift(a18, 48);
    { uint64_t t170 = a46; a46 = o_add(t170, a6); a6 = o_sub(t170, a6); }
    { uint64_t t171 = a2; a2 = o_add(t171, a18); a18 = o_sub(t171, a18); }
    { uint64_t t172 = a22; a22 = o_add(t172, a66); a66 = o_sub(t172, a66); }
    { uint64_t t173 = a62; a62 = o_add(t173, a50); a50 = o_sub(t173, a50); }
    a50 = o_shift(a50, 48);
    { uint64_t t174 = a22; a22 = o_add(t174, a62); a62 = o_sub(t174, a62); }
    { uint64_t t175 = a66; a66 = o_add(t175, a50); a50 = o_sub(t175, a50); }
    { uint64_t t176 = a54; a54 = o_add(t176, a26); a26 = o_sub(t176, a26); }
    { uint64_t t177 = a10; a10 = o_add(t177, a30); a30 = o_sub(t177, a30); }
    a30 = o_shift(a30, 48);
    { uint64_t t178 = a54; a54 = o_add(t178, a10); a10 = o_sub(t178, a10); }
    { uint64_t t179 = a26; a26 = o_add(t179, a30); a30 = o_sub(t179, a30); }
    a2 = o_shift(a2, 12);
    a6 = o_shift(a6, 24);
    a18 = o_shift(a18, 36);
    a66 = o_shift(a66, 24);
    a62 = o_shift(a62, 48);
    a50 = o_shift(a50, 72);
    a26 = o_shift(a26, 36);
    a10 = o_shift(a10, 72);
    a30 = o_neg(o_shift(a30, 12));
    { uint64_t t180 = a38; a38 = o_add(t180, a22); a22 = o_sub(t180, a22); }
    { uint64_t t181 = a46; a46 = o_add(t181, a54); a54 = o_sub(t181, a54); }
    a54 = o_shift(a54, 48);
    { uint64_t t182 = a38; a38 = o_add(t182, a46); a46 = o_sub(t182, a46); }
    { uint64_t t183 = a22; a22 = o_add(t183, a54); a54 = o_sub(t183, a54); }
    { uint64_t t184 = a58; a58 = o_add(t184, a66); a66 = o_sub(t184, a66); }
    { uint64_t t185 = a2; a2 = o_add(t185, a26); a26 = o_sub(t185, a26); }
    a26 = o_shift(a26, 48);
    { uint64_t t186 = a58; a58 = o_add(t186, a2); a2 = o_sub(t186, a2); }
    { uint64_t t187 = a66; a66 = o_add(t187, a26); a26 = o_sub(t187, a26); }
    { uint64_t t188 = a14; a14 = o_add(t188, a62); a62 = o_sub(t188, a62); }
    { uint64_t t189 = a6; a6 = o_add(t189, a10); a10 = o_sub(t189, a10); }
    a10 = o_shift(a10, 48);
    { uint64_t t190 = a14; a14 = o_add(t190, a6); a6 = o_sub(t190, a6); }
    { uint64_t t191 = a62; a62 = o_add(t191, a10); a10 = o_sub(t191, a10); }
    { uint64_t t192 = a42; a42 = o_add(t192, a50); a50 = o_sub(t192, a50); }
    { uint64_t t193 = a18; a18 = o_add(t193, a30); a30 = o_sub(t193, a30); }
    a30 = o_shift(a30, 48);
    { uint64_t t194 = a42; a42 = o_add(t194, a18); a18 = o_sub(t194, a18); }
    { uint64_t t195 = a50; a50 = o_add(t195, a30); a30 = o_sub(t195, a30); }
    { uint64_t t196 = a55; a55 = o_add(t196, a47); a47 = o_sub(t196, a47); }
    { uint64_t t197 = a67; a67 = o_add(t197, a35); a35 = o_sub(t197, a35); }
    a35 = o_shift(a35, 48);
    { uint64_t t198 = a55; a55 = o_add(t198, a67); a67 = o_sub(t198, a67); }
    { uint64_t t199 = a47; a47 = o_add(t199, a35); a35 = o_sub(t199, a35); }
    { uint64_t t200 = a7; a7 = o_add(t200, a27); a27 = o_sub(t200, a27); }
    { uint64_t t201 = a11; a11 = o_add(t201, a23); a23 = o_sub(t201, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t202 = a7; a7 = o_add(t202, a11); a11 = o_sub(t202, a11); }
    { uint64_t t203 = a27; a27 = o_add(t203, a23); a23 = o_sub(t203, a23); }
    { uint64_t t204 = a59; a59 = o_add(t204, a43); a43 = o_sub(t204, a43); }
    { uint64_t t205 = a15; a15 = o_add(t205, a19); a19 = o_sub(t205, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t206 = a59; a59 = o_add(t206, a15); a15 = o_sub(t206, a15); }
    { uint64_t t207 = a43; a43 = o_add(t207, a19); a19 = o_sub(t207, a19); }
    { uint64_t t208 = a31; a31 = o_add(t208, a3); a3 = o_sub(t208, a3); }
    { uint64_t t209 = a39; a39 = o_add(t209, a63); a63 = o_sub(t209, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t210 = a31; a31 = o_add(t210, a39); a39 = o_sub(t210, a39); }
    { uint64_t t211 = a3; a3 = o_add(t211, a63); a63 = o_sub(t211, a63); }
    a27 = o_shift(a27, 12);
    a11 = o_shift(a11, 24);
    a23 = o_shift(a23, 36);
    a43 = o_shift(a43, 24);
    a15 = o_shift(a15, 48);
    a19 = o_shift(a19, 72);
    a3 = o_shift(a3, 36);
    a39 = o_shift(a39, 72);
    a63 = o_neg(o_shift(a63, 12));
    { uint64_t t212 = a55; a55 = o_add(t212, a59); a59 = o_sub(t212, a59); }
    { uint64_t t213 = a7; a7 = o_add(t213, a31); a31 = o_sub(t213, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t214 = a55; a55 = o_add(t214, a7); a7 = o_sub(t214, a7); }
    { uint64_t t215 = a59; a59 = o_add(t215, a31); a31 = o_sub(t215, a31); }
    { uint64_t t216 = a47; a47 = o_add(t216, a43); a43 = o_sub(t216, a43); }
    { uint64_t t217 = a27; a27 = o_add(t217, a3); a3 = o_sub(t217, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t218 = a47; a47 = o_add(t218, a27); a27 = o_sub(t218, a27); }
    { uint64_t t219 = a43; a43 = o_add(t219, a3); a3 = o_sub(t219, a3); }
    { uint64_t t220 = a67; a67 = o_add(t220, a15); a15 = o_sub(t220, a15); }
    { uint64_t t221 = a11; a11 = o_add(t221, a39); a39 = o_sub(t221, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t222 = a67; a67 = o_add(t222, a11); a11 = o_sub(t222, a11); }
    { uint64_t t223 = a15; a15 = o_add(t223, a39); a39 = o_sub(t223, a39); }
    { uint64_t t224 = a35; a35 = o_add(t224, a19); a19 = o_sub(t224, a19); }
    { uint64_t t225 = a23; a23 = o_add(t225, a63); a63 = o_sub(t225, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t226 = a35; a35 = o_add(t226, a23); a23 = o_sub(t226, a23); }
    { uint64_t t227 = a19; a19 = o_add(t227, a63); a63 = o_sub(t227, a63); }
    uint64_t t228 = a51;
    a51 = o_add(a51, a55);
    a55 = o_mul(a55, 1152921504338411520ULL);
    a47 = o_mul(a47, 6259776822214049175ULL);
    a67 = o_mul(a67, 9380094172986290191ULL);
    a35 = o_mul(a35, 891943630314919127ULL);
    a59 = o_mul(a59, 17228171707553225791ULL);
    a43 = o_mul(a43, 12855743360534130886ULL);
    a15 = o_mul(a15, 6167687396920564837ULL);
    a19 = o_mul(a19, 17201834061724655524ULL);
    a7 = o_mul(a7, 15308299771656910737ULL);
    a27 = o_mul(a27, 18186005861103657533ULL);
    a11 = o_mul(a11, 53595491891823545ULL);
    a23 = o_mul(a23, 1906638201581172103ULL);
    a31 = o_mul(a31, 18303651001328874822ULL);
    a3 = o_mul(a3, 3077466521755967626ULL);
    a39 = o_mul(a39, 12423593102987598328ULL);
    a63 = o_mul(a63, 18361513053649472048ULL);
    a55 = o_add(a55, t228);
    { uint64_t t229 = a55; a55 = o_add(t229, a7); a7 = o_sub(t229, a7); }
    { uint64_t t230 = a31; a31 = o_add(t230, a59); a59 = o_sub(t230, a59); }
    a59 = o_shift(a59, 48);
    { uint64_t t231 = a55; a55 = o_add(t231, a31); a31 = o_sub(t231, a31); }
    { uint64_t t232 = a7; a7 = o_add(t232, a59); a59 = o_sub(t232, a59); }
    { uint64_t t233 = a63; a63 = o_add(t233, a19); a19 = o_sub(t233, a19); }
    { uint64_t t234 = a23; a23 = o_add(t234, a35); a35 = o_sub(t234, a35); }
    a35 = o_shift(a35, 48);
    { uint64_t t235 = a63; a63 = o_add(t235, a23); a23 = o_sub(t235, a23); }
    { uint64_t t236 = a19; a19 = o_add(t236, a35); a35 = o_sub(t236, a35); }
    { uint64_t t237 = a39; a39 = o_add(t237, a15); a15 = o_sub(t237, a15); }
    { uint64_t t238 = a11; a11 = o_add(t238, a67); a67 = o_sub(t238, a67); }
    a67 = o_shift(a67, 48);
    { uint64_t t239 = a39; a39 = o_add(t239, a11); a11 = o_sub(t239, a11); }
    { uint64_t t240 = a15; a15 = o_add(t240, a67); a67 = o_sub(t240, a67); }
    { uint64_t t241 = a3; a3 = o_add(t241, a43); a43 = o_sub(t241, a43); }
    { uint64_t t242 = a27; a27 = o_add(t242, a47); a47 = o_sub(t242, a47); }
    a47 = o_shift(a47, 48);
    { uint64_t t243 = a3; a3 = o_add(t243, a27); a27 = o_sub(t243, a27); }
    { uint64_t t244 = a43; a43 = o_add(t244, a47); a47 = o_sub(t244, a47); }
    a19 = o_shift(a19, 12);
    a23 = o_shift(a23, 24);
    a35 = o_shift(a35, 36);
    a15 = o_shift(a15, 24);
    a11 = o_shift(a11, 48);
    a67 = o_shift(a67, 72);
    a43 = o_shift(a43, 36);
    a27 = o_shift(a27, 72);
    a47 = o_neg(o_shift(a47, 12));
    { uint64_t t245 = a55; a55 = o_add(t245, a39); a39 = o_sub(t245, a39); }
    { uint64_t t246 = a63; a63 = o_add(t246, a3); a3 = o_sub(t246, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t247 = a55; a55 = o_add(t247, a63); a63 = o_sub(t247, a63); }
    { uint64_t t248 = a39; a39 = o_add(t248, a3); a3 = o_sub(t248, a3); }
    { uint64_t t249 = a7; a7 = o_add(t249, a15); a15 = o_sub(t249, a15); }
    { uint64_t t250 = a19; a19 = o_add(t250, a43); a43 = o_sub(t250, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t251 = a7; a7 = o_add(t251, a19); a19 = o_sub(t251, a19); }
    { uint64_t t252 = a15; a15 = o_add(t252, a43); a43 = o_sub(t252, a43); }
    { uint64_t t253 = a31; a31 = o_add(t253, a11); a11 = o_sub(t253, a11); }
    { uint64_t t254 = a23; a23 = o_add(t254, a27); a27 = o_sub(t254, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t255 = a31; a31 = o_add(t255, a23); a23 = o_sub(t255, a23); }
    { uint64_t t256 = a11; a11 = o_add(t256, a27); a27 = o_sub(t256, a27); }
    { uint64_t t257 = a59; a59 = o_add(t257, a67); a67 = o_sub(t257, a67); }
    { uint64_t t258 = a35; a35 = o_add(t258, a47); a47 = o_sub(t258, a47); }
    a47 = o_shift(a47, 48);
    { uint64_t t259 = a59; a59 = o_add(t259, a35); a35 = o_sub(t259, a35); }
    { uint64_t t260 = a67; a67 = o_add(t260, a47); a47 = o_sub(t260, a47); }
    { uint64_t t261 = a0; a0 = o_add(t261, a34); a34 = o_sub(t261, a34); }
    { uint64_t t262 = a17; a17 = o_add(t262, a51); a51 = o_sub(t262, a51); }
    a51 = o_shift(a51, 48);
    { uint64_t t263 = a0; a0 = o_add(t263, a17); a17 = o_sub(t263, a17); }
    { uint64_t t264 = a34; a34 = o_add(t264, a51); a51 = o_sub(t264, a51); }
    { uint64_t t265 = a4; a4 = o_add(t265, a38); a38 = o_sub(t265, a38); }
    { uint64_t t266 = a21; a21 = o_add(t266, a55); a55 = o_sub(t266, a55); }
    a55 = o_shift(a55, 48);
    { uint64_t t267 = a4; a4 = o_add(t267, a21); a21 = o_sub(t267, a21); }
    { uint64_t t268 = a38; a38 = o_add(t268, a55); a55 = o_sub(t268, a55); }
    { uint64_t t269 = a44; a44 = o_add(t269, a10); a10 = o_sub(t269, a10); }
    { uint64_t t270 = a61; a61 = o_add(t270, a27); a27 = o_sub(t270, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t271 = a44; a44 = o_add(t271, a61); a61 = o_sub(t271, a61); }
    { uint64_t t272 = a10; a10 = o_add(t272, a27); a27 = o_sub(t272, a27); }
    { uint64_t t273 = a24; a24 = o_add(t273, a58); a58 = o_sub(t273, a58); }
    { uint64_t t274 = a41; a41 = o_add(t274, a7); a7 = o_sub(t274, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t275 = a24; a24 = o_add(t275, a41); a41 = o_sub(t275, a41); }
    { uint64_t t276 = a58; a58 = o_add(t276, a7); a7 = o_sub(t276, a7); }
    { uint64_t t277 = a20; a20 = o_add(t277, a54); a54 = o_sub(t277, a54); }
    { uint64_t t278 = a37; a37 = o_add(t278, a3); a3 = o_sub(t278, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t279 = a20; a20 = o_add(t279, a37); a37 = o_sub(t279, a37); }
    { uint64_t t280 = a54; a54 = o_add(t280, a3); a3 = o_sub(t280, a3); }
    { uint64_t t281 = a32; a32 = o_add(t281, a66); a66 = o_sub(t281, a66); }
    { uint64_t t282 = a49; a49 = o_add(t282, a15); a15 = o_sub(t282, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t283 = a32; a32 = o_add(t283, a49); a49 = o_sub(t283, a49); }
    { uint64_t t284 = a66; a66 = o_add(t284, a15); a15 = o_sub(t284, a15); }
    { uint64_t t285 = a64; a64 = o_add(t285, a30); a30 = o_sub(t285, a30); }
    { uint64_t t286 = a13; a13 = o_add(t286, a47); a47 = o_sub(t286, a47); }
    a47 = o_shift(a47, 48);
    { uint64_t t287 = a64; a64 = o_add(t287, a13); a13 = o_sub(t287, a13); }
    { uint64_t t288 = a30; a30 = o_add(t288, a47); a47 = o_sub(t288, a47); }
    { uint64_t t289 = a52; a52 = o_add(t289, a18); a18 = o_sub(t289, a18); }
    { uint64_t t290 = a1; a1 = o_add(t290, a35); a35 = o_sub(t290, a35); }
    a35 = o_shift(a35, 48);
    { uint64_t t291 = a52; a52 = o_add(t291, a1); a1 = o_sub(t291, a1); }
    { uint64_t t292 = a18; a18 = o_add(t292, a35); a35 = o_sub(t292, a35); }
    { uint64_t t293 = a40; a40 = o_add(t293, a6); a6 = o_sub(t293, a6); }
    { uint64_t t294 = a57; a57 = o_add(t294, a23); a23 = o_sub(t294, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t295 = a40; a40 = o_add(t295, a57); a57 = o_sub(t295, a57); }
    { uint64_t t296 = a6; a6 = o_add(t296, a23); a23 = o_sub(t296, a23); }
    { uint64_t t297 = a48; a48 = o_add(t297, a14); a14 = o_sub(t297, a14); }
    { uint64_t t298 = a65; a65 = o_add(t298, a31); a31 = o_sub(t298, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t299 = a48; a48 = o_add(t299, a65); a65 = o_sub(t299, a65); }
    { uint64_t t300 = a14; a14 = o_add(t300, a31); a31 = o_sub(t300, a31); }
    { uint64_t t301 = a8; a8 = o_add(t301, a42); a42 = o_sub(t301, a42); }
    { uint64_t t302 = a25; a25 = o_add(t302, a59); a59 = o_sub(t302, a59); }
    a59 = o_shift(a59, 48);
    { uint64_t t303 = a8; a8 = o_add(t303, a25); a25 = o_sub(t303, a25); }
    { uint64_t t304 = a42; a42 = o_add(t304, a59); a59 = o_sub(t304, a59); }
    { uint64_t t305 = a16; a16 = o_add(t305, a50); a50 = o_sub(t305, a50); }
    { uint64_t t306 = a33; a33 = o_add(t306, a67); a67 = o_sub(t306, a67); }
    a67 = o_shift(a67, 48);
    { uint64_t t307 = a16; a16 = o_add(t307, a33); a33 = o_sub(t307, a33); }
    { uint64_t t308 = a50; a50 = o_add(t308, a67); a67 = o_sub(t308, a67); }
    { uint64_t t309 = a60; a60 = o_add(t309, a26); a26 = o_sub(t309, a26); }
    { uint64_t t310 = a9; a9 = o_add(t310, a43); a43 = o_sub(t310, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t311 = a60; a60 = o_add(t311, a9); a9 = o_sub(t311, a9); }
    { uint64_t t312 = a26; a26 = o_add(t312, a43); a43 = o_sub(t312, a43); }
    { uint64_t t313 = a56; a56 = o_add(t313, a22); a22 = o_sub(t313, a22); }
    { uint64_t t314 = a5; a5 = o_add(t314, a39); a39 = o_sub(t314, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t315 = a56; a56 = o_add(t315, a5); a5 = o_sub(t315, a5); }
    { uint64_t t316 = a22; a22 = o_add(t316, a39); a39 = o_sub(t316, a39); }
    { uint64_t t317 = a36; a36 = o_add(t317, a2); a2 = o_sub(t317, a2); }
    { uint64_t t318 = a53; a53 = o_add(t318, a19); a19 = o_sub(t318, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t319 = a36; a36 = o_add(t319, a53); a53 = o_sub(t319, a53); }
    { uint64_t t320 = a2; a2 = o_add(t320, a19); a19 = o_sub(t320, a19); }
    { uint64_t t321 = a28; a28 = o_add(t321, a62); a62 = o_sub(t321, a62); }
    { uint64_t t322 = a45; a45 = o_add(t322, a11); a11 = o_sub(t322, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t323 = a28; a28 = o_add(t323, a45); a45 = o_sub(t323, a45); }
    { uint64_t t324 = a62; a62 = o_add(t324, a11); a11 = o_sub(t324, a11); }
    { uint64_t t325 = a12; a12 = o_add(t325, a46); a46 = o_sub(t325, a46); }
    { uint64_t t326 = a29; a29 = o_add(t326, a63); a63 = o_sub(t326, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t327 = a12; a12 = o_add(t327, a29); a29 = o_sub(t327, a29); }
    { uint64_t t328 = a46; a46 = o_add(t328, a63); a63 = o_sub(t328, a63); }
    v[0] = a0;
    v[1] = a38;
    v[2] = a61;
    v[3] = a7;
    v[4] = a20;
    v[5] = a66;
    v[6] = a13;
    v[7] = a35;
    v[8] = a40;
    v[9] = a14;
    v[10] = a25;
    v[11] = a67;
    v[12] = a60;
    v[13] = a22;
    v[14] = a53;
    v[15] = a11;
    v[16] = a12;
    v[17] = a34;
    v[18] = a21;
    v[19] = a27;
    v[20] = a24;
    v[21] = a54;
    v[22] = a49;
    v[23] = a47;
    v[24] = a52;
    v[25] = a6;
    v[26] = a65;
    v[27] = a59;
    v[28] = a16;
    v[29] = a26;
    v[30] = a5;
    v[31] = a19;
    v[32] = a28;
    v[33] = a46;
    v[34] = a17;
    v[35] = a55;
    v[36] = a44;
    v[37] = a58;
    v[38] = a37;
    v[39] = a15;
    v[40] = a64;
    v[41] = a18;
    v[42] = a57;
    v[43] = a31;
    v[44] = a8;
    v[45] = a50;
    v[46] = a9;
    v[47] = a39;
    v[48] = a36;
    v[49] = a62;
    v[50] = a29;
    v[51] = a51;
    v[52] = a4;
    v[53] = a10;
    v[54] = a41;
    v[55] = a3;
    v[56] = a32;
    v[57] = a30;
    v[58] = a1;
    v[59] = a23;
    v[60] = a48;
    v[61] = a42;
    v[62] = a33;
    v[63] = a43;
    v[64] = a56;
    v[65] = a2;
    v[66] = a45;
    v[67] = a63;
}

static void o_ntt_80(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33], a34 = v[34], a35 = v[35], a36 = v[36], a37 = v[37], a38 = v[38], a39 = v[39], a40 = v[40], a41 = v[41], a42 = v[42], a43 = v[43], a44 = v[44], a45 = v[45], a46 = v[46], a47 = v[47], a48 = v[48], a49 = v[49], a50 = v[50], a51 = v[51], a52 = v[52], a53 = v[53], a54 = v[54], a55 = v[55], a56 = v[56], a57 = v[57], a58 = v[58], a59 = v[59], a60 = v[60], a61 = v[61], a62 = v[62], a63 = v[63], a64 = v[64], a65 = v[65], a66 = v[66], a67 = v[67], a68 = v[68], a69 = v[69], a70 = v[70], a71 = v[71], a72 = v[72], a73 = v[73], a74 = v[74], a75 = v[75], a76 = v[76], a77 = v[77], a78 = v[78], a79 = v[79];
    { uint64_t t1 = a0; a0 = o_add(t1, a40); a40 = o_sub(t1, a40); }
    { uint64_t t2 = a10; a10 = o_add(t2, a50); a50 = o_sub(t2, a50); }
    { uint64_t t3 = a20; a20 = o_add(t3, a60); a60 = o_sub(t3, a60); }
    { uint64_t t4 = a30; a30 = o_add(t4, a70); a70 = o_sub(t4, a70); }
    a50 = o_shift(a50, 24);
    a60 = o_shift(a60, 48);
    a70 = o_shift(a70, 72);
    { uint64_t t5 = a0; a0 = o_add(t5, a20); a20 = o_sub(t5, a20); }
    { uint64_t t6 = a10; a10 = o_add(t6, a30); a30 = o_sub(t6, a30); }
    a30 = o_shift(a30, 48);
    { uint64_t t7 = a0; a0 = o_add(t7, a10); a10 = o_sub(t7, a10); }
    { uint64_t t8 = a20; a20 = o_add(t8, a30); a30 = o_sub(t8, a30); }
    { uint64_t t9 = a40; a40 = o_add(t9, a60); a60 = o_sub(t9, a60); }
    { uint64_t t10 = a50; a50 = o_add(t10, a70); a70 = o_sub(t10, a70); }
    a70 = o_shift(a70, 48);
    { uint64_t t11 = a40; a40 = o_add(t11, a50); a50 = o_sub(t11, a50); }
    { uint64_t t12 = a60; a60 = o_add(t12, a70); a70 = o_sub(t12, a70); }
    { uint64_t t13 = a1; a1 = o_add(t13, a41); a41 = o_sub(t13, a41); }
    { uint64_t t14 = a11; a11 = o_add(t14, a51); a51 = o_sub(t14, a51); }
    { uint64_t t15 = a21; a21 = o_add(t15, a61); a61 = o_sub(t15, a61); }
    { uint64_t t16 = a31; a31 = o_add(t16, a71); a71 = o_sub(t16, a71); }
    a51 = o_shift(a51, 24);
    a61 = o_shift(a61, 48);
    a71 = o_shift(a71, 72);
    { uint64_t t17 = a1; a1 = o_add(t17, a21); a21 = o_sub(t17, a21); }
    { uint64_t t18 = a11; a11 = o_add(t18, a31); a31 = o_sub(t18, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t19 = a1; a1 = o_add(t19, a11); a11 = o_sub(t19, a11); }
    { uint64_t t20 = a21; a21 = o_add(t20, a31); a31 = o_sub(t20, a31); }
    { uint64_t t21 = a41; a41 = o_add(t21, a61); a61 = o_sub(t21, a61); }
    { uint64_t t22 = a51; a51 = o_add(t22, a71); a71 = o_sub(t22, a71); }
    a71 = o_shift(a71, 48);
    { uint64_t t23 = a41; a41 = o_add(t23, a51); a51 = o_sub(t23, a51); }
    { uint64_t t24 = a61; a61 = o_add(t24, a71); a71 = o_sub(t24, a71); }
    { uint64_t t25 = a2; a2 = o_add(t25, a42); a42 = o_sub(t25, a42); }
    { uint64_t t26 = a12; a12 = o_add(t26, a52); a52 = o_sub(t26, a52); }
    { uint64_t t27 = a22; a22 = o_add(t27, a62); a62 = o_sub(t27, a62); }
    { uint64_t t28 = a32; a32 = o_add(t28, a72); a72 = o_sub(t28, a72); }
    a52 = o_shift(a52, 24);
    a62 = o_shift(a62, 48);
    a72 = o_shift(a72, 72);
    { uint64_t t29 = a2; a2 = o_add(t29, a22); a22 = o_sub(t29, a22); }
    { uint64_t t30 = a12; a12 = o_add(t30, a32); a32 = o_sub(t30, a32); }
    a32 = o_shift(a32, 48);
    { uint64_t t31 = a2; a2 = o_add(t31, a12); a12 = o_sub(t31, a12); }
    { uint64_t t32 = a22; a22 = o_add(t32, a32); a32 = o_sub(t32, a32); }
    { uint64_t t33 = a42; a42 = o_add(t33, a62); a62 = o_sub(t33, a62); }
    { uint64_t t34 = a52; a52 = o_add(t34, a72); a72 = o_sub(t34, a72); }
    a72 = o_shift(a72, 48);
    { uint64_t t35 = a42; a42 = o_add(t35, a52); a52 = o_sub(t35, a52); }
    { uint64_t t36 = a62; a62 = o_add(t36, a72); a72 = o_sub(t36, a72); }
    { uint64_t t37 = a3; a3 = o_add(t37, a43); a43 = o_sub(t37, a43); }
    { uint64_t t38 = a13; a13 = o_add(t38, a53); a53 = o_sub(t38, a53); }
    { uint64_t t39 = a23; a23 = o_add(t39, a63); a63 = o_sub(t39, a63); }
    { uint64_t t40 = a33; a33 = o_add(t40, a73); a73 = o_sub(t40, a73); }
    a53 = o_shift(a53, 24);
    a63 = o_shift(a63, 48);
    a73 = o_shift(a73, 72);
    { uint64_t t41 = a3; a3 = o_add(t41, a23); a23 = o_sub(t41, a23); }
    { uint64_t t42 = a13; a13 = o_add(t42, a33); a33 = o_sub(t42, a33); }
    a33 = o_shift(a33, 48);
    { uint64_t t43 = a3; a3 = o_add(t43, a13); a13 = o_sub(t43, a13); }
    { uint64_t t44 = a23; a23 = o_add(t44, a33); a33 = o_sub(t44, a33); }
    { uint64_t t45 = a43; a43 = o_add(t45, a63); a63 = o_sub(t45, a63); }
    { uint64_t t46 = a53; a53 = o_add(t46, a73); a73 = o_sub(t46, a73); }
    a73 = o_shift(a73, 48);
    { uint64_t t47 = a43; a43 = o_add(t47, a53); a53 = o_sub(t47, a53); }
    { uint64_t t48 = a63; a63 = o_add(t48, a73); a73 = o_sub(t48, a73); }
    { uint64_t t49 = a4; a4 = o_add(t49, a44); a44 = o_sub(t49, a44); }
    { uint64_t t50 = a14; a14 = o_add(t50, a54); a54 = o_sub(t50, a54); }
    { uint64_t t51 = a24; a24 = o_add(t51, a64); a64 = o_sub(t51, a64); }
    { uint64_t t52 = a34; a34 = o_add(t52, a74); a74 = o_sub(t52, a74); }
    a54 = o_shift(a54, 24);
    a64 = o_shift(a64, 48);
    a74 = o_shift(a74, 72);
    { uint64_t t53 = a4; a4 = o_add(t53, a24); a24 = o_sub(t53, a24); }
    { uint64_t t54 = a14; a14 = o_add(t54, a34); a34 = o_sub(t54, a34); }
    a34 = o_shift(a34, 48);
    { uint64_t t55 = a4; a4 = o_add(t55, a14); a14 = o_sub(t55, a14); }
    { uint64_t t56 = a24; a24 = o_add(t56, a34); a34 = o_sub(t56, a34); }
    { uint64_t t57 = a44; a44 = o_add(t57, a64); a64 = o_sub(t57, a64); }
    { uint64_t t58 = a54; a54 = o_add(t58, a74); a74 = o_sub(t58, a74); }
    a74 = o_shift(a74, 48);
    { uint64_t t59 = a44; a44 = o_add(t59, a54); a54 = o_sub(t59, a54); }
    { uint64_t t60 = a64; a64 = o_add(t60, a74); a74 = o_sub(t60, a74); }
    { uint64_t t61 = a5; a5 = o_add(t61, a45); a45 = o_sub(t61, a45); }
    { uint64_t t62 = a15; a15 = o_add(t62, a55); a55 = o_sub(t62, a55); }
    { uint64_t t63 = a25; a25 = o_add(t63, a65); a65 = o_sub(t63, a65); }
    { uint64_t t64 = a35; a35 = o_add(t64, a75); a75 = o_sub(t64, a75); }
    a55 = o_shift(a55, 24);
    a65 = o_shift(a65, 48);
    a75 = o_shift(a75, 72);
    { uint64_t t65 = a5; a5 = o_add(t65, a25); a25 = o_sub(t65, a25); }
    { uint64_t t66 = a15; a15 = o_add(t66, a35); a35 = o_sub(t66, a35); }
    a35 = o_shift(a35, 48);
    { uint64_t t67 = a5; a5 = o_add(t67, a15); a15 = o_sub(t67, a15); }
    { uint64_t t68 = a25; a25 = o_add(t68, a35); a35 = o_sub(t68, a35); }
    { uint64_t t69 = a45; a45 = o_add(t69, a65); a65 = o_sub(t69, a65); }
    { uint64_t t70 = a55; a55 = o_add(t70, a75); a75 = o_sub(t70, a75); }
    a75 = o_shift(a75, 48);
    { uint64_t t71 = a45; a45 = o_add(t71, a55); a55 = o_sub(t71, a55); }
    { uint64_t t72 = a65; a65 = o_add(t72, a75); a75 = o_sub(t72, a75); }
    { uint64_t t73 = a6; a6 = o_add(t73, a46); a46 = o_sub(t73, a46); }
    { uint64_t t74 = a16; a16 = o_add(t74, a56); a56 = o_sub(t74, a56); }
    { uint64_t t75 = a26; a26 = o_add(t75, a66); a66 = o_sub(t75, a66); }
    { uint64_t t76 = a36; a36 = o_add(t76, a76); a76 = o_sub(t76, a76); }
    a56 = o_shift(a56, 24);
    a66 = o_shift(a66, 48);
    a76 = o_shift(a76, 72);
    { uint64_t t77 = a6; a6 = o_add(t77, a26); a26 = o_sub(t77, a26); }
    { uint64_t t78 = a16; a16 = o_add(t78, a36); a36 = o_sub(t78, a36); }
    a36 = o_shift(a36, 48);
    { uint64_t t79 = a6; a6 = o_add(t79, a16); a16 = o_sub(t79, a16); }
    { uint64_t t80 = a26; a26 = o_add(t80, a36); a36 = o_sub(t80, a36); }
    { uint64_t t81 = a46; a46 = o_add(t81, a66); a66 = o_sub(t81, a66); }
    { uint64_t t82 = a56; a56 = o_add(t82, a76); a76 = o_sub(t82, a76); }
    a76 = o_shift(a76, 48);
    { uint64_t t83 = a46; a46 = o_add(t83, a56); a56 = o_sub(t83, a56); }
    { uint64_t t84 = a66; a66 = o_add(t84, a76); a76 = o_sub(t84, a76); }
    { uint64_t t85 = a7; a7 = o_add(t85, a47); a47 = o_sub(t85, a47); }
    { uint64_t t86 = a17; a17 = o_add(t86, a57); a57 = o_sub(t86, a57); }
    { uint64_t t87 = a27; a27 = o_add(t87, a67); a67 = o_sub(t87, a67); }
    { uint64_t t88 = a37; a37 = o_add(t88, a77); a77 = o_sub(t88, a77); }
    a57 = o_shift(a57, 24);
    a67 = o_shift(a67, 48);
    a77 = o_shift(a77, 72);
    { uint64_t t89 = a7; a7 = o_add(t89, a27); a27 = o_sub(t89, a27); }
    { uint64_t t90 = a17; a17 = o_add(t90, a37); a37 = o_sub(t90, a37); }
    a37 = o_shift(a37, 48);
    { uint64_t t91 = a7; a7 = o_add(t91, a17); a17 = o_sub(t91, a17); }
    { uint64_t t92 = a27; a27 = o_add(t92, a37); a37 = o_sub(t92, a37); }
    { uint64_t t93 = a47; a47 = o_add(t93, a67); a67 = o_sub(t93, a67); }
    { uint64_t t94 = a57; a57 = o_add(t94, a77); a77 = o_sub(t94, a77); }
    a77 = o_shift(a77, 48);
    { uint64_t t95 = a47; a47 = o_add(t95, a57); a57 = o_sub(t95, a57); }
    { uint64_t t96 = a67; a67 = o_add(t96, a77); a77 = o_sub(t96, a77); }
    { uint64_t t97 = a8; a8 = o_add(t97, a48); a48 = o_sub(t97, a48); }
    { uint64_t t98 = a18; a18 = o_add(t98, a58); a58 = o_sub(t98, a58); }
    { uint64_t t99 = a28; a28 = o_add(t99, a68); a68 = o_sub(t99, a68); }
    { uint64_t t100 = a38; a38 = o_add(t100, a78); a78 = o_sub(t100, a78); }
    a58 = o_shift(a58, 24);
    a68 = o_shift(a68, 48);
    a78 = o_shift(a78, 72);
    { uint64_t t101 = a8; a8 = o_add(t101, a28); a28 = o_sub(t101, a28); }
    { uint64_t t102 = a18; a18 = o_add(t102, a38); a38 = o_sub(t102, a38); }
    a38 = o_shift(a38, 48);
    { uint64_t t103 = a8; a8 = o_add(t103, a18); a18 = o_sub(t103, a18); }
    { uint64_t t104 = a28; a28 = o_add(t104, a38); a38 = o_sub(t104, a38); }
    { uint64_t t105 = a48; a48 = o_add(t105, a68); a68 = o_sub(t105, a68); }
    { uint64_t t106 = a58; a58 = o_add(t106, a78); a78 = o_sub(t106, a78); }
    a78 = o_shift(a78, 48);
    { uint64_t t107 = a48; a48 = o_add(t107, a58); a58 = o_sub(t107, a58); }
    { uint64_t t108 = a68; a68 = o_add(t108, a78); a78 = o_sub(t108, a78); }
    { uint64_t t109 = a9; a9 = o_add(t109, a49); a49 = o_sub(t109, a49); }
    { uint64_t t110 = a19; a19 = o_add(t110, a59); a59 = o_sub(t110, a59); }
    { uint64_t t111 = a29; a29 = o_add(t111, a69); a69 = o_sub(t111, a69); }
    { uint64_t t112 = a39; a39 = o_add(t112, a79); a79 = o_sub(t112, a79); }
    a59 = o_shift(a59, 24);
    a69 = o_shift(a69, 48);
    a79 = o_shift(a79, 72);
    { uint64_t t113 = a9; a9 = o_add(t113, a29); a29 = o_sub(t113, a29); }
    { uint64_t t114 = a19; a19 = o_add(t114, a39); a39 = o_sub(t114, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t115 = a9; a9 = o_add(t115, a19); a19 = o_sub(t115, a19); }
    { uint64_t t116 = a29; a29 = o_add(t116, a39); a39 = o_sub(t116, a39); }
    { uint64_t t117 = a49; a49 = o_add(t117, a69); a69 = o_sub(t117, a69); }
    { uint64_t t118 = a59; a59 = o_add(t118, a79); a79 = o_sub(t118, a79); }
    a79 = o_shift(a79, 48);
    { uint64_t t119 = a49; a49 = o_add(t119, a59); a59 = o_sub(t119, a59); }
    { uint64_t t120 = a69; a69 = o_add(t120, a79); a79 = o_sub(t120, a79); }
    a41 = o_mul(a41, 6193879297194861051ULL);
    a21 = o_mul(a21, 9148693690730647261ULL);
    a61 = o_mul(a61, 2598525327269793995ULL);
    a11 = o_mul(a11, 5290193119087387221ULL);
    a51 = o_shift(a51, 12);
    a31 = o_mul(a31, 5856505865097423521ULL);
    a71 = o_mul(a71, 7712152251710425105ULL);
    a42 = o_mul(a42, 9148693690730647261ULL);
    a22 = o_mul(a22, 5290193119087387221ULL);
    a62 = o_mul(a62, 5856505865097423521ULL);
    a12 = o_mul(a12, 18235156514275634624ULL);
    a52 = o_shift(a52, 24);
    a32 = o_mul(a32, 8149776168132872528ULL);
    a72 = o_mul(a72, 11331573348451128694ULL);
    a43 = o_mul(a43, 2598525327269793995ULL);
    a23 = o_mul(a23, 5856505865097423521ULL);
    a63 = o_mul(a63, 12153478289216064362ULL);
    a13 = o_mul(a13, 8149776168132872528ULL);
    a53 = o_shift(a53, 36);
    a33 = o_mul(a33, 4419751934697861046ULL);
    a73 = o_mul(a73, 3918829805224079129ULL);
    a44 = o_mul(a44, 5290193119087387221ULL);
    a24 = o_mul(a24, 18235156514275634624ULL);
    a64 = o_mul(a64, 8149776168132872528ULL);
    a14 = o_mul(a14, 1041288259238279555ULL);
    a54 = o_shift(a54, 48);
    a34 = o_mul(a34, 17073700798457888299ULL);
    a74 = o_mul(a74, 17869255328328231396ULL);
    a45 = o_shift(a45, 12);
    a25 = o_shift(a25, 24);
    a65 = o_shift(a65, 36);
    a15 = o_shift(a15, 48);
    a55 = o_shift(a55, 60);
    a35 = o_shift(a35, 72);
    a75 = o_shift(a75, 84);
    a46 = o_mul(a46, 5856505865097423521ULL);
    a26 = o_mul(a26, 8149776168132872528ULL);
    a66 = o_mul(a66, 4419751934697861046ULL);
    a16 = o_mul(a16, 17073700798457888299ULL);
    a56 = o_shift(a56, 72);
    a36 = o_mul(a36, 2281812832982421726ULL);
    a76 = o_mul(a76, 9298050378683937060ULL);
    a47 = o_mul(a47, 7712152251710425105ULL);
    a27 = o_mul(a27, 11331573348451128694ULL);
    a67 = o_mul(a67, 3918829805224079129ULL);
    a17 = o_mul(a17, 17869255328328231396ULL);
    a57 = o_shift(a57, 84);
    a37 = o_mul(a37, 9298050378683937060ULL);
    a77 = o_mul(a77, 6293265780198519959ULL);
    a48 = o_mul(a48, 18235156514275634624ULL);
    a28 = o_mul(a28, 1041288259238279555ULL);
    a68 = o_mul(a68, 17073700798457888299ULL);
    a18 = o_mul(a18, 15820824984080659046ULL);
    a58 = o_neg(a58);
    a38 = o_mul(a38, 211587555138949697ULL);
    a78 = o_mul(a78, 17405455810176304766ULL);
    a49 = o_mul(a49, 12153478289216064362ULL);
    a29 = o_mul(a29, 4419751934697861046ULL);
    a69 = o_mul(a69, 15685396404952554508ULL);
    a19 = o_mul(a19, 2281812832982421726ULL);
    a59 = o_neg(o_shift(a59, 12));
    a39 = o_mul(a39, 7115170720963455627ULL);
    a79 = o_mul(a79, 11398751642682958806ULL);
    { uint64_t t121 = a2; a2 = o_add(t121, a8); a8 = o_sub(t121, a8); }
    { uint64_t t122 = a6; a6 = o_add(t122, a4); a4 = o_sub(t122, a4); }
    a4 = o_shift(a4, 48);
    { uint64_t t123 = a2; a2 = o_add(t123, a6); a6 = o_sub(t123, a6); }
    { uint64_t t124 = a8; a8 = o_add(t124, a4); a4 = o_sub(t124, a4); }
    uint64_t t125 = a0;
    a0 = o_add(a0, a2);
    a2 = o_mul(a2, 4611686017353646080ULL);
    a8 = o_mul(a8, 16181989089180173841ULL);
    a6 = o_mul(a6, 5818851782451133869ULL);
    a4 = o_mul(a4, 11322249509082494407ULL);
    a2 = o_add(a2, t125);
    { uint64_t t126 = a2; a2 = o_add(t126, a6); a6 = o_sub(t126, a6); }
    { uint64_t t127 = a4; a4 = o_add(t127, a8); a8 = o_sub(t127, a8); }
    a8 = o_shift(a8, 48);
    { uint64_t t128 = a2; a2 = o_add(t128, a4); a4 = o_sub(t128, a4); }
    { uint64_t t129 = a6; a6 = o_add(t129, a8); a8 = o_sub(t129, a8); }
    { uint64_t t130 = a7; a7 = o_add(t130, a3); a3 = o_sub(t130, a3); }
    { uint64_t t131 = a1; a1 = o_add(t131, a9); a9 = o_sub(t131, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t132 = a7; a7 = o_add(t132, a1); a1 = o_sub(t132, a1); }
    { uint64_t t133 = a3; a3 = o_add(t133, a9); a9 = o_sub(t133, a9); }
    uint64_t t134 = a5;
    a5 = o_add(a5, a7);
    a7 = o_mul(a7, 4611686017353646080ULL);
    a3 = o_mul(a3, 16181989089180173841ULL);
    a1 = o_mul(a1, 5818851782451133869ULL);
    a9 = o_mul(a9, 11322249509082494407ULL);
    a7 = o_add(a7, t134);
    { uint64_t t135 = a7; a7 = o_add(t135, a1); a1 = o_sub(t135, a1); }
    { uint64_t t136 = a9; a9 = o_add(t136, a3); a3 = o_sub(t136, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t137 = a7; a7 = o_add(t137, a9); a9 = o_sub(t137, a9); }
    { uint64_t t138 = a1; a1 = o_add(t138, a3); a3 = o_sub(t138, a3); }
    { uint64_t t139 = a0; a0 = o_add(t139, a5); a5 = o_sub(t139, a5); }
    { uint64_t t140 = a2; a2 = o_add(t140, a7); a7 = o_sub(t140, a7); }
    { uint64_t t141 = a6; a6 = o_add(t141, a1); a1 = o_sub(t141, a1); }
    { uint64_t t142 = a8; a8 = o_add(t142, a3); a3 = o_sub(t142, a3); }
    { uint64_t t143 = a4; a4 = o_add(t143, a9); a9 = o_sub(t143, a9); }
    { uint64_t t144 = a42; a42 = o_add(t144, a48); a48 = o_sub(t144, a48); }
    { uint64_t t145 = a46; a46 = o_add(t145, a44); a44 = o_sub(t145, a44); }
    a44 = o_shift(a44, 48);
    { uint64_t t146 = a42; a42 = o_add(t146, a46); a46 = o_sub(t146, a46); }
    { uint64_t t147 = a48; a48 = o_add(t147, a44); a44 = o_sub(t147, a44); }
    uint64_t t148 = a40;
    a40 = o_add(a40, a42);
    a42 = o_mul(a42, 4611686017353646080ULL);
    a48 = o_mul(a48, 16181989089180173841ULL);
    a46 = o_mul(a46, 5818851782451133869ULL);
    a44 = o_mul(a44, 11322249509082494407ULL);
    a42 = o_add(a42, t148);
    { uint64_t t149 = a42; a42 = o_add(t149, a46); a46 = o_sub(t149, a46); }
    { uint64_t t150 = a44; a44 = o_add(t150, a48); a48 = o_sub(t150, a48); }
    a48 = o_shift(a48, 48);
    { uint64_t t151 = a42; a42 = o_add(t151, a44); a44 = o_sub(t151, a44); }
    { uint64_t t152 = a46; a46 = o_add(t152, a48); a48 = o_sub(t152, a48); }
    { uint64_t t153 = a47; a47 = o_add(t153, a43); a43 = o_sub(t153, a43); }
    { uint64_t t154 = a41; a41 = o_add(t154, a49); a49 = o_sub(t154, a49); }
    a49 = o_shift(a49, 48);
    { uint64_t t155 = a47; a47 = o_add(t155, a41); a41 = o_sub(t155, a41); }
    { uint64_t t156 = a43; a43 = o_add(t156, a49); a49 = o_sub(t156, a49); }
    uint64_t t157 = a45;
    a45 = o_add(a45, a47);
    a47 = o_mul(a47, 4611686017353646080ULL);
    a43 = o_mul(a43, 16181989089180173841ULL);
    a41 = o_mul(a41, 5818851782451133869ULL);
    a49 = o_mul(a49, 11322249509082494407ULL);
    a47 = o_add(a47, t157);
    { uint64_t t158 = a47; a47 = o_add(t158, a41); a41 = o_sub(t158, a41); }
    { uint64_t t159 = a49; a49 = o_add(t159, a43); a43 = o_sub(t159, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t160 = a47; a47 = o_add(t160, a49); a49 = o_sub(t160, a49); }
    { uint64_t t161 = a41; a41 = o_add(t161, a43); a43 = o_sub(t161, a43); }
    { uint64_t t162 = a40; a40 = o_add(t162, a45); a45 = o_sub(t162, a45); }
    { uint64_t t163 = a42; a42 = o_add(t163, a47); a47 = o_sub(t163, a47); }
    { uint64_t t164 = a46; a46 = o_add(t164, a41); a41 = o_sub(t164, a41); }
    { uint64_t t165 = a48; a48 = o_add(t165, a43); a43 = o_sub(t165, a43); }
    { uint64_t t166 = a44; a44 = o_add(t166, a49); a49 = o_sub(t166, a49); }
    { uint64_t t167 = a22; a22 = o_add(t167, a28); a28 = o_sub(t167, a28); }
    { uint64_t t168 = a26; a26 = o_add(t168, a24); a24 = o_sub(t168, a24); }
    a24 = o_shift(a24, 48);
    { uint64_t t169 = a22; a22 = o_add(t169, a26); a26 = o_sub(t169, a26); }
    { uint64_t t170 = a28; a28 = o_add(t170, a24); a24 = o_sub(t170, a24); }
    uint64_t t171 = a20;
    a20 = o_add(a20, a22);
    a22 = o_mul(a22, 4611686017353646080ULL);
    a28 = o_mul(a28, 16181989089180173841ULL);
    a26 = o_mul(a26, 5818851782451133869ULL);
    a24 = o_mul(a24, 11322249509082494407ULL);
    a22 = o_add(a22, t171);
    { uint64_t t172 = a22; a22 = o_add(t172, a26); a26 = o_sub(t172, a26); }
    { uint64_t t173 = a24; a24 = o_add(t173, a28); a28 = o_sub(t173, a28); }
    a28 = o_shift(a28, 48);
    { uint64_t t174 = a22; a22 = o_add(t174, a24); a24 = o_sub(t174, a24); }
    { uint64_t t175 = a26; a26 = o_add(t175, a28); a28 = o_sub(t175, a28); }
    { uint64_t t176 = a27; a27 = o_add(t176, a23); a23 = o_sub(t176, a23); }
    { uint64_t t177 = a21; a21 = o_add(t177, a29); a29 = o_sub(t177, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t178 = a27; a27 = o_add(t178, a21); a21 = o_sub(t178, a21); }
    { uint64_t t179 = a23; a23 = o_add(t179, a29); a29 = o_sub(t179, a29); }
    uint64_t t180 = a25;
    a25 = o_add(a25, a27);
    a27 = o_mul(a27, 4611686017353646080ULL);
    a23 = o_mul(a23, 16181989089180173841ULL);
    a21 = o_mul(a21, 5818851782451133869ULL);
    a29 = o_mul(a29, 11322249509082494407ULL);
    a27 = o_add(a27, t180);
    { uint64_t t181 = a27; a27 = o_add(t181, a21); a21 = o_sub(t181, a21); }
    { uint64_t t182 = a29; a29 = o_add(t182, a23); a23 = o_sub(t182, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t183 = a27; a27 = o_add(t183, a29); a29 = o_sub(t183, a29); }
    { uint64_t t184 = a21; a21 = o_add(t184, a23); a23 = o_sub(t184, a23); }
    { uint64_t t185 = a20; a20 = o_add(t185, a25); a25 = o_sub(t185, a25); }
    { uint64_t t186 = a22; a22 = o_add(t186, a27); a27 = o_sub(t186, a27); }
    { uint64_t t187 = a26; a26 = o_add(t187, a21); a21 = o_sub(t187, a21); }
    { uint64_t t188 = a28; a28 = o_add(t188, a23); a23 = o_sub(t188, a23); }
    { uint64_t t189 = a24; a24 = o_add(t189, a29); a29 = o_sub(t189, a29); }
    { uint64_t t190 = a62; a62 = o_add(t190, a68); a68 = o_sub(t190, a68); }
    { uint64_t t191 = a66; a66 = o_add(t191, a64); a64 = o_sub(t191, a64); }
    a64 = o_shift(a64, 48);
    { uint64_t t192 = a62; a62 = o_add(t192, a66); a66 = o_sub(t192, a66); }
    { uint64_t t193 = a68; a68 = o_add(t193, a64); a64 = o_sub(t193, a64); }
    uint64_t t194 = a60;
    a60 = o_add(a60, a62);
    a62 = o_mul(a62, 4611686017353646080ULL);
    a68 = o_mul(a68, 16181989089180173841ULL);
    a66 = o_mul(a66, 5818851782451133869ULL);
    a64 = o_mul(a64, 11322249509082494407ULL);
    a62 = o_add(a62, t194);
    { uint64_t t195 = a62; a62 = o_add(t195, a66); a66 = o_sub(t195, a66); }
    { uint64_t t196 = a64; a64 = o_add(t196, a68); a68 = o_sub(t196, a68); }
    a68 = o_shift(a68, 48);
    { uint64_t t197 = a62; a62 = o_add(t197, a64); a64 = o_sub(t197, a64); }
    { uint64_t t198 = a66; a66 = o_add(t198, a68); a68 = o_sub(t198, a68); }
    { uint64_t t199 = a67; a67 = o_add(t199, a63); a63 = o_sub(t199, a63); }
    { uint64_t t200 = a61; a61 = o_add(t200, a69); a69 = o_sub(t200, a69); }
    a69 = o_shift(a69, 48);
    { uint64_t t201 = a67; a67 = o_add(t201, a61); a61 = o_sub(t201, a61); }
    { uint64_t t202 = a63; a63 = o_add(t202, a69); a69 = o_sub(t202, a69); }
    uint64_t t203 = a65;
    a65 = o_add(a65, a67);
    a67 = o_mul(a67, 4611686017353646080ULL);
    a63 = o_mul(a63, 16181989089180173841ULL);
    a61 = o_mul(a61, 5818851782451133869ULL);
    a69 = o_mul(a69, 11322249509082494407ULL);
    a67 = o_add(a67, t203);
    { uint64_t t204 = a67; a67 = o_add(t204, a61); a61 = o_sub(t204, a61); }
    { uint64_t t205 = a69; a69 = o_add(t205, a63); a63 = o_sub(t205, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t206 = a67; a67 = o_add(t206, a69); a69 = o_sub(t206, a69); }
    { uint64_t t207 = a61; a61 = o_add(t207, a63); a63 = o_sub(t207, a63); }
    { uint64_t t208 = a60; a60 = o_add(t208, a65); a65 = o_sub(t208, a65); }
    { uint64_t t209 = a62; a62 = o_add(t209, a67); a67 = o_sub(t209, a67); }
    { uint64_t t210 = a66; a66 = o_add(t210, a61); a61 = o_sub(t210, a61); }
    { uint64_t t211 = a68; a68 = o_add(t211, a63); a63 = o_sub(t211, a63); }
    { uint64_t t212 = a64; a64 = o_add(t212, a69); a69 = o_sub(t212, a69); }
    { uint64_t t213 = a12; a12 = o_add(t213, a18); a18 = o_sub(t213, a18); }
    { uint64_t t214 = a16; a16 = o_add(t214, a14); a14 = o_sub(t214, a14); }
    a14 = o_shift(a14, 48);
    { uint64_t t215 = a12; a12 = o_add(t215, a16); a16 = o_sub(t215, a16); }
    { uint64_t t216 = a18; a18 = o_add(t216, a14); a14 = o_sub(t216, a14); }
    uint64_t t217 = a10;
    a10 = o_add(a10, a12);
    a12 = o_mul(a12, 4611686017353646080ULL);
    a18 = o_mul(a18, 16181989089180173841ULL);
    a16 = o_mul(a16, 5818851782451133869ULL);
    a14 = o_mul(a14, 11322249509082494407ULL);
    a12 = o_add(a12, t217);
    { uint64_t t218 = a12; a12 = o_add(t218, a16); a16 = o_sub(t218, a16); }
    { uint64_t t219 = a14; a14 = o_add(t219, a18); a18 = o_sub(t219, a18); }
    a18 = o_shift(a18, 48);
    { uint64_t t220 = a12; a12 = o_add(t220, a14); a14 = o_sub(t220, a14); }
    { uint64_t t221 = a16; a16 = o_add(t221, a18); a18 = o_sub(t221, a18); }
    { uint64_t t222 = a17; a17 = o_add(t222, a13); a13 = o_sub(t222, a13); }
    { uint64_t t223 = a11; a11 = o_add(t223, a19); a19 = o_sub(t223, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t224 = a17; a17 = o_add(t224, a11); a11 = o_sub(t224, a11); }
    { uint64_t t225 = a13; a13 = o_add(t225, a19); a19 = o_sub(t225, a19); }
    uint64_t t226 = a15;
    a15 = o_add(a15, a17);
    a17 = o_mul(a17, 4611686017353646080ULL);
    a13 = o_mul(a13, 16181989089180173841ULL);
    a11 = o_mul(a11, 5818851782451133869ULL);
    a19 = o_mul(a19, 11322249509082494407ULL);
    a17 = o_add(a17, t226);
    { uint64_t t227 = a17; a17 = o_add(t227, a11); a11 = o_sub(t227, a11); }
    { uint64_t t228 = a19; a19 = o_add(t228, a13); a13 = o_sub(t228, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t229 = a17; a17 = o_add(t229, a19); a19 = o_sub(t229, a19); }
    { uint64_t t230 = a11; a11 = o_add(t230, a13); a13 = o_sub(t230, a13); }
    { uint64_t t231 = a10; a10 = o_add(t231, a15); a15 = o_sub(t231, a15); }
    { uint64_t t232 = a12; a12 = o_add(t232, a17); a17 = o_sub(t232, a17); }
    { uint64_t t233 = a16; a16 = o_add(t233, a11); a11 = o_sub(t233, a11); }
    { uint64_t t234 = a18; a18 = o_add(t234, a13); a13 = o_sub(t234, a13); }
    { uint64_t t235 = a14; a14 = o_add(t235, a19); a19 = o_sub(t235, a19); }
    { uint64_t t236 = a52; a52 = o_add(t236, a58); a58 = o_sub(t236, a58); }
    { uint64_t t237 = a56; a56 = o_add(t237, a54); a54 = o_sub(t237, a54); }
    a54 = o_shift(a54, 48);
    { uint64_t t238 = a52; a52 = o_add(t238, a56); a56 = o_sub(t238, a56); }
    { uint64_t t239 = a58; a58 = o_add(t239, a54); a54 = o_sub(t239, a54); }
    uint64_t t240 = a50;
    a50 = o_add(a50, a52);
    a52 = o_mul(a52, 4611686017353646080ULL);
    a58 = o_mul(a58, 16181989089180173841ULL);
    a56 = o_mul(a56, 5818851782451133869ULL);
    a54 = o_mul(a54, 11322249509082494407ULL);
    a52 = o_add(a52, t240);
    { uint64_t t241 = a52; a52 = o_add(t241, a56); a56 = o_sub(t241, a56); }
    { uint64_t t242 = a54; a54 = o_add(t242, a58); a58 = o_sub(t242, a58); }
    a58 = o_shift(a58, 48);
    { uint64_t t243 = a52; a52 = o_add(t243, a54); a54 = o_sub(t243, a54); }
    { uint64_t t244 = a56; a56 = o_add(t244, a58); a58 = o_sub(t244, a58); }
    { uint64_t t245 = a57; a57 = o_add(t245, a53); a53 = o_sub(t245, a53); }
    { uint64_t t246 = a51; a51 = o_add(t246, a59); a59 = o_sub(t246, a59); }
    a59 = o_shift(a59, 48);
    { uint64_t t247 = a57; a57 = o_add(t247, a51); a51 = o_sub(t247, a51); }
    { uint64_t t248 = a53; a53 = o_add(t248, a59); a59 = o_sub(t248, a59); }
    uint64_t t249 = a55;
    a55 = o_add(a55, a57);
    a57 = o_mul(a57, 4611686017353646080ULL);
    a53 = o_mul(a53, 16181989089180173841ULL);
    a51 = o_mul(a51, 5818851782451133869ULL);
    a59 = o_mul(a59, 11322249509082494407ULL);
    a57 = o_add(a57, t249);
    { uint64_t t250 = a57; a57 = o_add(t250, a51); a51 = o_sub(t250, a51); }
    { uint64_t t251 = a59; a59 = o_add(t251, a53); a53 = o_sub(t251, a53); }
    a53 = o_shift(a53, 48);
    { uint64_t t252 = a57; a57 = o_add(t252, a59); a59 = o_sub(t252, a59); }
    { uint64_t t253 = a51; a51 = o_add(t253, a53); a53 = o_sub(t253, a53); }
    { uint64_t t254 = a50; a50 = o_add(t254, a55); a55 = o_sub(t254, a55); }
    { uint64_t t255 = a52; a52 = o_add(t255, a57); a57 = o_sub(t255, a57); }
    { uint64_t t256 = a56; a56 = o_add(t256, a51); a51 = o_sub(t256, a51); }
    { uint64_t t257 = a58; a58 = o_add(t257, a53); a53 = o_sub(t257, a53); }
    { uint64_t t258 = a54; a54 = o_add(t258, a59); a59 = o_sub(t258, a59); }
    { uint64_t t259 = a32; a32 = o_add(t259, a38); a38 = o_sub(t259, a38); }
    { uint64_t t260 = a36; a36 = o_add(t260, a34); a34 = o_sub(t260, a34); }
    a34 = o_shift(a34, 48);
    { uint64_t t261 = a32; a32 = o_add(t261, a36); a36 = o_sub(t261, a36); }
    { uint64_t t262 = a38; a38 = o_add(t262, a34); a34 = o_sub(t262, a34); }
    uint64_t t263 = a30;
    a30 = o_add(a30, a32);
    a32 = o_mul(a32, 4611686017353646080ULL);
    a38 = o_mul(a38, 16181989089180173841ULL);
    a36 = o_mul(a36, 5818851782451133869ULL);
    a34 = o_mul(a34, 11322249509082494407ULL);
    a32 = o_add(a32, t263);
    { uint64_t t264 = a32; a32 = o_add(t264, a36); a36 = o_sub(t264, a36); }
    { uint64_t t265 = a34; a34 = o_add(t265, a38); a38 = o_sub(t265, a38); }
    a38 = o_shift(a38, 48);
    { uint64_t t266 = a32; a32 = o_add(t266, a34); a34 = o_sub(t266, a34); }
    { uint64_t t267 = a36; a36 = o_add(t267, a38); a38 = o_sub(t267, a38); }
    { uint64_t t268 = a37; a37 = o_add(t268, a33); a33 = o_sub(t268, a33); }
    { uint64_t t269 = a31; a31 = o_add(t269, a39); a39 = o_sub(t269, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t270 = a37; a37 = o_add(t270, a31); a31 = o_sub(t270, a31); }
    { uint64_t t271 = a33; a33 = o_add(t271, a39); a39 = o_sub(t271, a39); }
    uint64_t t272 = a35;
    a35 = o_add(a35, a37);
    a37 = o_mul(a37, 4611686017353646080ULL);
    a33 = o_mul(a33, 16181989089180173841ULL);
    a31 = o_mul(a31, 5818851782451133869ULL);
    a39 = o_mul(a39, 11322249509082494407ULL);
    a37 = o_add(a37, t272);
    { uint64_t t273 = a37; a37 = o_add(t273, a31); a31 = o_sub(t273, a31); }
    { uint64_t t274 = a39; a39 = o_add(t274, a33); a33 = o_sub(t274, a33); }
    a33 = o_shift(a33, 48);
    { uint64_t t275 = a37; a37 = o_add(t275, a39); a39 = o_sub(t275, a39); }
    { uint64_t t276 = a31; a31 = o_add(t276, a33); a33 = o_sub(t276, a33); }
    { uint64_t t277 = a30; a30 = o_add(t277, a35); a35 = o_sub(t277, a35); }
    { uint64_t t278 = a32; a32 = o_add(t278, a37); a37 = o_sub(t278, a37); }
    { uint64_t t279 = a36; a36 = o_add(t279, a31); a31 = o_sub(t279, a31); }
    { uint64_t t280 = a38; a38 = o_add(t280, a33); a33 = o_sub(t280, a33); }
    { uint64_t t281 = a34; a34 = o_add(t281, a39); a39 = o_sub(t281, a39); }
    { uint64_t t282 = a72; a72 = o_add(t282, a78); a78 = o_sub(t282, a78); }
    { uint64_t t283 = a76; a76 = o_add(t283, a74); a74 = o_sub(t283, a74); }
    a74 = o_shift(a74, 48);
    { uint64_t t284 = a72; a72 = o_add(t284, a76); a76 = o_sub(t284, a76); }
    { uint64_t t285 = a78; a78 = o_add(t285, a74); a74 = o_sub(t285, a74); }
    uint64_t t286 = a70;
    a70 = o_add(a70, a72);
    a72 = o_mul(a72, 4611686017353646080ULL);
    a78 = o_mul(a78, 16181989089180173841ULL);
    a76 = o_mul(a76, 5818851782451133869ULL);
    a74 = o_mul(a74, 11322249509082494407ULL);
    a72 = o_add(a72, t286);
    { uint64_t t287 = a72; a72 = o_add(t287, a76); a76 = o_sub(t287, a76); }
    { uint64_t t288 = a74; a74 = o_add(t288, a78); a78 = o_sub(t288, a78); }
    a78 = o_shift(a78, 48);
    { uint64_t t289 = a72; a72 = o_add(t289, a74); a74 = o_sub(t289, a74); }
    { uint64_t t290 = a76; a76 = o_add(t290, a78); a78 = o_sub(t290, a78); }
    { uint64_t t291 = a77; a77 = o_add(t291, a73); a73 = o_sub(t291, a73); }
    { uint64_t t292 = a71; a71 = o_add(t292, a79); a79 = o_sub(t292, a79); }
    a79 = o_shift(a79, 48);
    { uint64_t t293 = a77; a77 = o_add(t293, a71); a71 = o_sub(t293, a71); }
    { uint64_t t294 = a73; a73 = o_add(t294, a79); a79 = o_sub(t294, a79); }
    uint64_t t295 = a75;
    a75 = o_add(a75, a77);
    a77 = o_mul(a77, 4611686017353646080ULL);
    a73 = o_mul(a73, 16181989089180173841ULL);
    a71 = o_mul(a71, 5818851782451133869ULL);
    a79 = o_mul(a79, 11322249509082494407ULL);
    a77 = o_add(a77, t295);
    { uint64_t t296 = a77; a77 = o_add(t296, a71); a71 = o_sub(t296, a71); }
    { uint64_t t297 = a79; a79 = o_add(t297, a73); a73 = o_sub(t297, a73); }
    a73 = o_shift(a73, 48);
    { uint64_t t298 = a77; a77 = o_add(t298, a79); a79 = o_sub(t298, a79); }
    { uint64_t t299 = a71; a71 = o_add(t299, a73); a73 = o_sub(t299, a73); }
    { uint64_t t300 = a70; a70 = o_add(t300, a75); a75 = o_sub(t300, a75); }
    { uint64_t t301 = a72; a72 = o_add(t301, a77); a77 = o_sub(t301, a77); }
    { uint64_t t302 = a76; a76 = o_add(t302, a71); a71 = o_sub(t302, a71); }
    { uint64_t t303 = a78; a78 = o_add(t303, a73); a73 = o_sub(t303, a73); }
    { uint64_t t304 = a74; a74 = o_add(t304, a79); a79 = o_sub(t304, a79); }
    v[0] = a0;
    v[1] = a40;
    v[2] = a20;
    v[3] = a60;
    v[4] = a10;
    v[5] = a50;
    v[6] = a30;
    v[7] = a70;
    v[8] = a7;
    v[9] = a47;
    v[10] = a27;
    v[11] = a67;
    v[12] = a17;
    v[13] = a57;
    v[14] = a37;
    v[15] = a77;
    v[16] = a6;
    v[17] = a46;
    v[18] = a26;
    v[19] = a66;
    v[20] = a16;
    v[21] = a56;
    v[22] = a36;
    v[23] = a76;
    v[24] = a3;
    v[25] = a43;
    v[26] = a23;
    v[27] = a63;
    v[28] = a13;
    v[29] = a53;
    v[30] = a33;
    v[31] = a73;
    v[32] = a4;
    v[33] = a44;
    v[34] = a24;
    v[35] = a64;
    v[36] = a14;
    v[37] = a54;
    v[38] = a34;
    v[39] = a74;
    v[40] = a5;
    v[41] = a45;
    v[42] = a25;
    v[43] = a65;
    v[44] = a15;
    v[45] = a55;
    v[46] = a35;
    v[47] = a75;
    v[48] = a2;
    v[49] = a42;
    v[50] = a22;
    v[51] = a62;
    v[52] = a12;
    v[53] = a52;
    v[54] = a32;
    v[55] = a72;
    v[56] = a1;
    v[57] = a41;
    v[58] = a21;
    v[59] = a61;
    v[60] = a11;
    v[61] = a51;
    v[62] = a31;
    v[63] = a71;
    v[64] = a8;
    v[65] = a48;
    v[66] = a28;
    v[67] = a68;
    v[68] = a18;
    v[69] = a58;
    v[70] = a38;
    v[71] = a78;
    v[72] = a9;
    v[73] = a49;
    v[74] = a29;
    v[75] = a69;
    v[76] = a19;
    v[77] = a59;
    v[78] = a39;
    v[79] = a79;
}

static void o_ntt_85(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33], a34 = v[34], a35 = v[35], a36 = v[36], a37 = v[37], a38 = v[38], a39 = v[39], a40 = v[40], a41 = v[41], a42 = v[42], a43 = v[43], a44 = v[44], a45 = v[45], a46 = v[46], a47 = v[47], a48 = v[48], a49 = v[49], a50 = v[50], a51 = v[51], a52 = v[52], a53 = v[53], a54 = v[54], a55 = v[55], a56 = v[56], a57 = v[57], a58 = v[58], a59 = v[59], a60 = v[60], a61 = v[61], a62 = v[62], a63 = v[63], a64 = v[64], a65 = v[65], a66 = v[66], a67 = v[67], a68 = v[68], a69 = v[69], a70 = v[70], a71 = v[71], a72 = v[72], a73 = v[73], a74 = v[74], a75 = v[75], a76 = v[76], a77 = v[77], a78 = v[78], a79 = v[79], a80 = v[80], a81 = v[81], a82 = v[82], a83 = v[83], a84 = v[84];
    { uint64_t t1 = a5; a5 = o_add(t1, a80); a80 = o_sub(t1, a80); }
    { uint64_t t2 = a20; a20 = o_add(t2, a65); a65 = o_sub(t2, a65); }
    a65 = o_shift(a65, 48);
    { uint64_t t3 = a5; a5 = o_add(t3, a20); a20 = o_sub(t3, a20); }
    { uint64_t t4 = a80; a80 = o_add(t4, a65); a65 = o_sub(t4, a65); }
    { uint64_t t5 = a30; a30 = o_add(t5, a55); a55 = o_sub(t5, a55); }
    { uint64_t t6 = a35; a35 = o_add(t6, a50); a50 = o_sub(t6, a50); }
    a50 = o_shift(a50, 48);
    { uint64_t t7 = a30; a30 = o_add(t7, a35); a35 = o_sub(t7, a35); }
    { uint64_t t8 = a55; a55 = o_add(t8, a50); a50 = o_sub(t8, a50); }
    { uint64_t t9 = a10; a10 = o_add(t9, a75); a75 = o_sub(t9, a75); }
    { uint64_t t10 = a40; a40 = o_add(t10, a45); a45 = o_sub(t10, a45); }
    a45 = o_shift(a45, 48);
    { uint64_t t11 = a10; a10 = o_add(t11, a40); a40 = o_sub(t11, a40); }
    { uint64_t t12 = a75; a75 = o_add(t12, a45); a45 = o_sub(t12, a45); }
    { uint64_t t13 = a60; a60 = o_add(t13, a25); a25 = o_sub(t13, a25); }
    { uint64_t t14 = a70; a70 = o_add(t14, a15); a15 = o_sub(t14, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t15 = a60; a60 = o_add(t15, a70); a70 = o_sub(t15, a70); }
    { uint64_t t16 = a25; a25 = o_add(t16, a15); a15 = o_sub(t16, a15); }
    a55 = o_shift(a55, 12);
    a35 = o_shift(a35, 24);
    a50 = o_shift(a50, 36);
    a75 = o_shift(a75, 24);
    a40 = o_shift(a40, 48);
    a45 = o_shift(a45, 72);
    a25 = o_shift(a25, 36);
    a70 = o_shift(a70, 72);
    a15 = o_neg(o_shift(a15, 12));
    { uint64_t t17 = a5; a5 = o_add(t17, a10); a10 = o_sub(t17, a10); }
    { uint64_t t18 = a30; a30 = o_add(t18, a60); a60 = o_sub(t18, a60); }
    a60 = o_shift(a60, 48);
    { uint64_t t19 = a5; a5 = o_add(t19, a30); a30 = o_sub(t19, a30); }
    { uint64_t t20 = a10; a10 = o_add(t20, a60); a60 = o_sub(t20, a60); }
    { uint64_t t21 = a80; a80 = o_add(t21, a75); a75 = o_sub(t21, a75); }
    { uint64_t t22 = a55; a55 = o_add(t22, a25); a25 = o_sub(t22, a25); }
    a25 = o_shift(a25, 48);
    { uint64_t t23 = a80; a80 = o_add(t23, a55); a55 = o_sub(t23, a55); }
    { uint64_t t24 = a75; a75 = o_add(t24, a25); a25 = o_sub(t24, a25); }
    { uint64_t t25 = a20; a20 = o_add(t25, a40); a40 = o_sub(t25, a40); }
    { uint64_t t26 = a35; a35 = o_add(t26, a70); a70 = o_sub(t26, a70); }
    a70 = o_shift(a70, 48);
    { uint64_t t27 = a20; a20 = o_add(t27, a35); a35 = o_sub(t27, a35); }
    { uint64_t t28 = a40; a40 = o_add(t28, a70); a70 = o_sub(t28, a70); }
    { uint64_t t29 = a65; a65 = o_add(t29, a45); a45 = o_sub(t29, a45); }
    { uint64_t t30 = a50; a50 = o_add(t30, a15); a15 = o_sub(t30, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t31 = a65; a65 = o_add(t31, a50); a50 = o_sub(t31, a50); }
    { uint64_t t32 = a45; a45 = o_add(t32, a15); a15 = o_sub(t32, a15); }
    uint64_t t33 = a0;
    a0 = o_add(a0, a5);
    a5 = o_mul(a5, 1152921504338411520ULL);
    a80 = o_mul(a80, 6259776822214049175ULL);
    a20 = o_mul(a20, 9380094172986290191ULL);
    a65 = o_mul(a65, 891943630314919127ULL);
    a10 = o_mul(a10, 17228171707553225791ULL);
    a75 = o_mul(a75, 12855743360534130886ULL);
    a40 = o_mul(a40, 6167687396920564837ULL);
    a45 = o_mul(a45, 17201834061724655524ULL);
    a30 = o_mul(a30, 15308299771656910737ULL);
    a55 = o_mul(a55, 18186005861103657533ULL);
    a35 = o_mul(a35, 53595491891823545ULL);
    a50 = o_mul(a50, 1906638201581172103ULL);
    a60 = o_mul(a60, 18303651001328874822ULL);
    a25 = o_mul(a25, 3077466521755967626ULL);
    a70 = o_mul(a70, 12423593102987598328ULL);
    a15 = o_mul(a15, 18361513053649472048ULL);
    a5 = o_add(a5, t33);
    { uint64_t t34 = a5; a5 = o_add(t34, a30); a30 = o_sub(t34, a30); }
    { uint64_t t35 = a60; a60 = o_add(t35, a10); a10 = o_sub(t35, a10); }
    a10 = o_shift(a10, 48);
    { uint64_t t36 = a5; a5 = o_add(t36, a60); a60 = o_sub(t36, a60); }
    { uint64_t t37 = a30; a30 = o_add(t37, a10); a10 = o_sub(t37, a10); }
    { uint64_t t38 = a15; a15 = o_add(t38, a45); a45 = o_sub(t38, a45); }
    { uint64_t t39 = a50; a50 = o_add(t39, a65); a65 = o_sub(t39, a65); }
    a65 = o_shift(a65, 48);
    { uint64_t t40 = a15; a15 = o_add(t40, a50); a50 = o_sub(t40, a50); }
    { uint64_t t41 = a45; a45 = o_add(t41, a65); a65 = o_sub(t41, a65); }
    { uint64_t t42 = a70; a70 = o_add(t42, a40); a40 = o_sub(t42, a40); }
    { uint64_t t43 = a35; a35 = o_add(t43, a20); a20 = o_sub(t43, a20); }
    a20 = o_shift(a20, 48);
    { uint64_t t44 = a70; a70 = o_add(t44, a35); a35 = o_sub(t44, a35); }
    { uint64_t t45 = a40; a40 = o_add(t45, a20); a20 = o_sub(t45, a20); }
    { uint64_t t46 = a25; a25 = o_add(t46, a75); a75 = o_sub(t46, a75); }
    { uint64_t t47 = a55; a55 = o_add(t47, a80); a80 = o_sub(t47, a80); }
    a80 = o_shift(a80, 48);
    { uint64_t t48 = a25; a25 = o_add(t48, a55); a55 = o_sub(t48, a55); }
    { uint64_t t49 = a75; a75 = o_add(t49, a80); a80 = o_sub(t49, a80); }
    a45 = o_shift(a45, 12);
    a50 = o_shift(a50, 24);
    a65 = o_shift(a65, 36);
    a40 = o_shift(a40, 24);
    a35 = o_shift(a35, 48);
    a20 = o_shift(a20, 72);
    a75 = o_shift(a75, 36);
    a55 = o_shift(a55, 72);
    a80 = o_neg(o_shift(a80, 12));
    { uint64_t t50 = a5; a5 = o_add(t50, a70); a70 = o_sub(t50, a70); }
    { uint64_t t51 = a15; a15 = o_add(t51, a25); a25 = o_sub(t51, a25); }
    a25 = o_shift(a25, 48);
    { uint64_t t52 = a5; a5 = o_add(t52, a15); a15 = o_sub(t52, a15); }
    { uint64_t t53 = a70; a70 = o_add(t53, a25); a25 = o_sub(t53, a25); }
    { uint64_t t54 = a30; a30 = o_add(t54, a40); a40 = o_sub(t54, a40); }
    { uint64_t t55 = a45; a45 = o_add(t55, a75); a75 = o_sub(t55, a75); }
    a75 = o_shift(a75, 48);
    { uint64_t t56 = a30; a30 = o_add(t56, a45); a45 = o_sub(t56, a45); }
    { uint64_t t57 = a40; a40 = o_add(t57, a75); a75 = o_sub(t57, a75); }
    { uint64_t t58 = a60; a60 = o_add(t58, a35); a35 = o_sub(t58, a35); }
    { uint64_t t59 = a50; a50 = o_add(t59, a55); a55 = o_sub(t59, a55); }
    a55 = o_shift(a55, 48);
    { uint64_t t60 = a60; a60 = o_add(t60, a50); a50 = o_sub(t60, a50); }
    { uint64_t t61 = a35; a35 = o_add(t61, a55); a55 = o_sub(t61, a55); }
    { uint64_t t62 = a10; a10 = o_add(t62, a20); a20 = o_sub(t62, a20); }
    { uint64_t t63 = a65; a65 = o_add(t63, a80); a80 = o_sub(t63, a80); }
    a80 = o_shift(a80, 48);
    { uint64_t t64 = a10; a10 = o_add(t64, a65); a65 = o_sub(t64, a65); }
    { uint64_t t65 = a20; a20 = o_add(t65, a80); a80 = o_sub(t65, a80); }
    { uint64_t t66 = a22; a22 = o_add(t66, a12); a12 = o_sub(t66, a12); }
    { uint64_t t67 = a37; a37 = o_add(t67, a82); a82 = o_sub(t67, a82); }
    a82 = o_shift(a82, 48);
    { uint64_t t68 = a22; a22 = o_add(t68, a37); a37 = o_sub(t68, a37); }
    { uint64_t t69 = a12; a12 = o_add(t69, a82); a82 = o_sub(t69, a82); }
    { uint64_t t70 = a47; a47 = o_add(t70, a72); a72 = o_sub(t70, a72); }
    { uint64_t t71 = a52; a52 = o_add(t71, a67); a67 = o_sub(t71, a67); }
    a67 = o_shift(a67, 48);
    { uint64_t t72 = a47; a47 = o_add(t72, a52); a52 = o_sub(t72, a52); }
    { uint64_t t73 = a72; a72 = o_add(t73, a67); a67 = o_sub(t73, a67); }
    { uint64_t t74 = a27; a27 = o_add(t74, a7); a7 = o_sub(t74, a7); }
    { uint64_t t75 = a57; a57 = o_add(t75, a62); a62 = o_sub(t75, a62); }
    a62 = o_shift(a62, 48);
    { uint64_t t76 = a27; a27 = o_add(t76, a57); a57 = o_sub(t76, a57); }
    { uint64_t t77 = a7; a7 = o_add(t77, a62); a62 = o_sub(t77, a62); }
    { uint64_t t78 = a77; a77 = o_add(t78, a42); a42 = o_sub(t78, a42); }
    { uint64_t t79 = a2; a2 = o_add(t79, a32); a32 = o_sub(t79, a32); }
    a32 = o_shift(a32, 48);
    { uint64_t t80 = a77; a77 = o_add(t80, a2); a2 = o_sub(t80, a2); }
    { uint64_t t81 = a42; a42 = o_add(t81, a32); a32 = o_sub(t81, a32); }
    a72 = o_shift(a72, 12);
    a52 = o_shift(a52, 24);
    a67 = o_shift(a67, 36);
    a7 = o_shift(a7, 24);
    a57 = o_shift(a57, 48);
    a62 = o_shift(a62, 72);
    a42 = o_shift(a42, 36);
    a2 = o_shift(a2, 72);
    a32 = o_neg(o_shift(a32, 12));
    { uint64_t t82 = a22; a22 = o_add(t82, a27); a27 = o_sub(t82, a27); }
    { uint64_t t83 = a47; a47 = o_add(t83, a77); a77 = o_sub(t83, a77); }
    a77 = o_shift(a77, 48);
    { uint64_t t84 = a22; a22 = o_add(t84, a47); a47 = o_sub(t84, a47); }
    { uint64_t t85 = a27; a27 = o_add(t85, a77); a77 = o_sub(t85, a77); }
    { uint64_t t86 = a12; a12 = o_add(t86, a7); a7 = o_sub(t86, a7); }
    { uint64_t t87 = a72; a72 = o_add(t87, a42); a42 = o_sub(t87, a42); }
    a42 = o_shift(a42, 48);
    { uint64_t t88 = a12; a12 = o_add(t88, a72); a72 = o_sub(t88, a72); }
    { uint64_t t89 = a7; a7 = o_add(t89, a42); a42 = o_sub(t89, a42); }
    { uint64_t t90 = a37; a37 = o_add(t90, a57); a57 = o_sub(t90, a57); }
    { uint64_t t91 = a52; a52 = o_add(t91, a2); a2 = o_sub(t91, a2); }
    a2 = o_shift(a2, 48);
    { uint64_t t92 = a37; a37 = o_add(t92, a52); a52 = o_sub(t92, a52); }
    { uint64_t t93 = a57; a57 = o_add(t93, a2); a2 = o_sub(t93, a2); }
    { uint64_t t94 = a82; a82 = o_add(t94, a62); a62 = o_sub(t94, a62); }
    { uint64_t t95 = a67; a67 = o_add(t95, a32); a32 = o_sub(t95, a32); }
    a32 = o_shift(a32, 48);
    { uint64_t t96 = a82; a82 = o_add(t96, a67); a67 = o_sub(t96, a67); }
    { uint64_t t97 = a62; a62 = o_add(t97, a32); a32 = o_sub(t97, a32); }
    uint64_t t98 = a17;
    a17 = o_add(a17, a22);
    a22 = o_mul(a22, 1152921504338411520ULL);
    a12 = o_mul(a12, 6259776822214049175ULL);
    a37 = o_mul(a37, 9380094172986290191ULL);
    a82 = o_mul(a82, 891943630314919127ULL);
    a27 = o_mul(a27, 17228171707553225791ULL);
    a7 = o_mul(a7, 12855743360534130886ULL);
    a57 = o_mul(a57, 6167687396920564837ULL);
    a62 = o_mul(a62, 17201834061724655524ULL);
    a47 = o_mul(a47, 15308299771656910737ULL);
    a72 = o_mul(a72, 18186005861103657533ULL);
    a52 = o_mul(a52, 53595491891823545ULL);
    a67 = o_mul(a67, 1906638201581172103ULL);
    a77 = o_mul(a77, 18303651001328874822ULL);
    a42 = o_mul(a42, 3077466521755967626ULL);
    a2 = o_mul(a2, 12423593102987598328ULL);
    a32 = o_mul(a32, 18361513053649472048ULL);
    a22 = o_add(a22, t98);
    { uint64_t t99 = a22; a22 = o_add(t99, a47); a47 = o_sub(t99, a47); }
    { uint64_t t100 = a77; a77 = o_add(t100, a27); a27 = o_sub(t100, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t101 = a22; a22 = o_add(t101, a77); a77 = o_sub(t101, a77); }
    { uint64_t t102 = a47; a47 = o_add(t102, a27); a27 = o_sub(t102, a27); }
    { uint64_t t103 = a32; a32 = o_add(t103, a62); a62 = o_sub(t103, a62); }
    { uint64_t t104 = a67; a67 = o_add(t104, a82); a82 = o_sub(t104, a82); }
    a82 = o_shift(a82, 48);
    { uint64_t t105 = a32; a32 = o_add(t105, a67); a67 = o_sub(t105, a67); }
    { uint64_t t106 = a62; a62 = o_add(t106, a82); a82 = o_sub(t106, a82); }
    { uint64_t t107 = a2; a2 = o_add(t107, a57); a57 = o_sub(t107, a57); }
    { uint64_t t108 = a52; a52 = o_add(t108, a37); a37 = o_sub(t108, a37); }
    a37 = o_shift(a37, 48);
    { uint64_t t109 = a2; a2 = o_add(t109, a52); a52 = o_sub(t109, a52); }
    { uint64_t t110 = a57; a57 = o_add(t110, a37); a37 = o_sub(t110, a37); }
    { uint64_t t111 = a42; a42 = o_add(t111, a7); a7 = o_sub(t111, a7); }
    { uint64_t t112 = a72; a72 = o_add(t112, a12); a12 = o_sub(t112, a12); }
    a12 = o_shift(a12, 48);
    { uint64_t t113 = a42; a42 = o_add(t113, a72); a72 = o_sub(t113, a72); }
    { uint64_t t114 = a7; a7 = o_add(t114, a12); a12 = o_sub(t114, a12); }
    a62 = o_shift(a62, 12);
    a67 = o_shift(a67, 24);
    a82 = o_shift(a82, 36);
    a57 = o_shift(a57, 24);
    a52 = o_shift(a52, 48);
    a37 = o_shift(a37, 72);
    a7 = o_shift(a7, 36);
    a72 = o_shift(a72, 72);
    a12 = o_neg(o_shift(a12, 12));
    { uint64_t t115 = a22; a22 = o_add(t115, a2); a2 = o_sub(t115, a2); }
    { uint64_t t116 = a32; a32 = o_add(t116, a42); a42 = o_sub(t116, a42); }
    a42 = o_shift(a42, 48);
    { uint64_t t117 = a22; a22 = o_add(t117, a32); a32 = o_sub(t117, a32); }
    { uint64_t t118 = a2; a2 = o_add(t118, a42); a42 = o_sub(t118, a42); }
    { uint64_t t119 = a47; a47 = o_add(t119, a57); a57 = o_sub(t119, a57); }
    { uint64_t t120 = a62; a62 = o_add(t120, a7); a7 = o_sub(t120, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t121 = a47; a47 = o_add(t121, a62); a62 = o_sub(t121, a62); }
    { uint64_t t122 = a57; a57 = o_add(t122, a7); a7 = o_sub(t122, a7); }
    { uint64_t t123 = a77; a77 = o_add(t123, a52); a52 = o_sub(t123, a52); }
    { uint64_t t124 = a67; a67 = o_add(t124, a72); a72 = o_sub(t124, a72); }
    a72 = o_shift(a72, 48);
    { uint64_t t125 = a77; a77 = o_add(t125, a67); a67 = o_sub(t125, a67); }
    { uint64_t t126 = a52; a52 = o_add(t126, a72); a72 = o_sub(t126, a72); }
    { uint64_t t127 = a27; a27 = o_add(t127, a37); a37 = o_sub(t127, a37); }
    { uint64_t t128 = a82; a82 = o_add(t128, a12); a12 = o_sub(t128, a12); }
    a12 = o_shift(a12, 48);
    { uint64_t t129 = a27; a27 = o_add(t129, a82); a82 = o_sub(t129, a82); }
    { uint64_t t130 = a37; a37 = o_add(t130, a12); a12 = o_sub(t130, a12); }
    { uint64_t t131 = a39; a39 = o_add(t131, a29); a29 = o_sub(t131, a29); }
    { uint64_t t132 = a54; a54 = o_add(t132, a14); a14 = o_sub(t132, a14); }
    a14 = o_shift(a14, 48);
    { uint64_t t133 = a39; a39 = o_add(t133, a54); a54 = o_sub(t133, a54); }
    { uint64_t t134 = a29; a29 = o_add(t134, a14); a14 = o_sub(t134, a14); }
    { uint64_t t135 = a64; a64 = o_add(t135, a4); a4 = o_sub(t135, a4); }
    { uint64_t t136 = a69; a69 = o_add(t136, a84); a84 = o_sub(t136, a84); }
    a84 = o_shift(a84, 48);
    { uint64_t t137 = a64; a64 = o_add(t137, a69); a69 = o_sub(t137, a69); }
    { uint64_t t138 = a4; a4 = o_add(t138, a84); a84 = o_sub(t138, a84); }
    { uint64_t t139 = a44; a44 = o_add(t139, a24); a24 = o_sub(t139, a24); }
    { uint64_t t140 = a74; a74 = o_add(t140, a79); a79 = o_sub(t140, a79); }
    a79 = o_shift(a79, 48);
    { uint64_t t141 = a44; a44 = o_add(t141, a74); a74 = o_sub(t141, a74); }
    { uint64_t t142 = a24; a24 = o_add(t142, a79); a79 = o_sub(t142, a79); }
    { uint64_t t143 = a9; a9 = o_add(t143, a59); a59 = o_sub(t143, a59); }
    { uint64_t t144 = a19; a19 = o_add(t144, a49); a49 = o_sub(t144, a49); }
    a49 = o_shift(a49, 48);
    { uint64_t t145 = a9; a9 = o_add(t145, a19); a19 = o_sub(t145, a19); }
    { uint64_t t146 = a59; a59 = o_add(t146, a49); a49 = o_sub(t146, a49); }
    a4 = o_shift(a4, 12);
    a69 = o_shift(a69, 24);
    a84 = o_shift(a84, 36);
    a24 = o_shift(a24, 24);
    a74 = o_shift(a74, 48);
    a79 = o_shift(a79, 72);
    a59 = o_shift(a59, 36);
    a19 = o_shift(a19, 72);
    a49 = o_neg(o_shift(a49, 12));
    { uint64_t t147 = a39; a39 = o_add(t147, a44); a44 = o_sub(t147, a44); }
    { uint64_t t148 = a64; a64 = o_add(t148, a9); a9 = o_sub(t148, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t149 = a39; a39 = o_add(t149, a64); a64 = o_sub(t149, a64); }
    { uint64_t t150 = a44; a44 = o_add(t150, a9); a9 = o_sub(t150, a9); }
    { uint64_t t151 = a29; a29 = o_add(t151, a24); a24 = o_sub(t151, a24); }
    { uint64_t t152 = a4; a4 = o_add(t152, a59); a59 = o_sub(t152, a59); }
    a59 = o_shift(a59, 48);
    { uint64_t t153 = a29; a29 = o_add(t153, a4); a4 = o_sub(t153, a4); }
    { uint64_t t154 = a24; a24 = o_add(t154, a59); a59 = o_sub(t154, a59); }
    { uint64_t t155 = a54; a54 = o_add(t155, a74); a74 = o_sub(t155, a74); }
    { uint64_t t156 = a69; a69 = o_add(t156, a19); a19 = o_sub(t156, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t157 = a54; a54 = o_add(t157, a69); a69 = o_sub(t157, a69); }
    { uint64_t t158 = a74; a74 = o_add(t158, a19); a19 = o_sub(t158, a19); }
    { uint64_t t159 = a14; a14 = o_add(t159, a79); a79 = o_sub(t159, a79); }
    { uint64_t t160 = a84; a84 = o_add(t160, a49); a49 = o_sub(t160, a49); }
    a49 = o_shift(a49, 48);
    { uint64_t t161 = a14; a14 = o_add(t161, a84); a84 = o_sub(t161, a84); }
    { uint64_t t162 = a79; a79 = o_add(t162, a49); a49 = o_sub(t162, a49); }
    uint64_t t163 = a34;
    a34 = o_add(a34, a39);
    a39 = o_mul(a39, 1152921504338411520ULL);
    a29 = o_mul(a29, 6259776822214049175ULL);
    a54 = o_mul(a54, 9380094172986290191ULL);
    a14 = o_mul(a14, 891943630314919127ULL);
    a44 = o_mul(a44, 17228171707553225791ULL);
    a24 = o_mul(a24, 12855743360534130886ULL);
    a74 = o_mul(a74, 6167687396920564837ULL);
    a79 = o_mul(a79, 17201834061724655524ULL);
    a64 = o_mul(a64, 15308299771656910737ULL);
    a4 = o_mul(a4, 18186005861103657533ULL);
    a69 = o_mul(a69, 53595491891823545ULL);
    a84 = o_mul(a84, 1906638201581172103ULL);
    a9 = o_mul(a9, 18303651001328874822ULL);
    a59 = o_mul(a59, 3077466521755967626ULL);
    a19 = o_mul(a19, 12423593102987598328ULL);
    a49 = o_mul(a49, 18361513053649472048ULL);
    a39 = o_add(a39, t163);
    { uint64_t t164 = a39; a39 = o_add(t164, a64); a64 = o_sub(t164, a64); }
    { uint64_t t165 = a9; a9 = o_add(t165, a44); a44 = o_sub(t165, a44); }
    a44 = o_shift(a44, 48);
    { uint64_t t166 = a39; a39 = o_add(t166, a9); a9 = o_sub(t166, a9); }
    { uint64_t t167 = a64; a64 = o_add(t167, a44); a44 = o_sub(t167, a44); }
    { uint64_t t168 = a49; a49 = o_add(t168, a79); a79 = o_sub(t168, a79); }
    { uint64_t t169 = a84; a84 = o_add(t169, a14); a14 = o_sub(t169, a14); }
    a14 = o_shift(a14, 48);
    { uint64_t t170 = a49; a49 = o_add(t170, a84); a84 = o_sub(t170, a84); }
    { uint64_t t171 = a79; a79 = o_add(t171, a14); a14 = o_sub(t171, a14); }
    { uint64_t t172 = a19; a19 = o_add(t172, a74); a74 = o_sub(t172, a74); }
    { uint64_t t173 = a69; a69 = o_add(t173, a54); a54 = o_sub(t173, a54); }
    a54 = o_shift(a54, 48);
    { uint64_t t174 = a19; a19 = o_add(t174, a69); a69 = o_sub(t174, a69); }
    { uint64_t t175 = a74; a74 = o_add(t175, a54); a54 = o_sub(t175, a54); }
    { uint64_t t176 = a59; a59 = o_add(t176, a24); a24 = o_sub(t176, a24); }
    { uint64_t t177 = a4; a4 = o_add(t177, a29); a29 = o_sub(t177, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t178 = a59; a59 = o_add(t178, a4); a4 = o_sub(t178, a4); }
    { uint64_t t179 = a24; a24 = o_add(t179, a29); a29 = o_sub(t179, a29); }
    a79 = o_shift(a79, 12);
    a84 = o_shift(a84, 24);
    a14 = o_shift(a14, 36);
    a74 = o_shift(a74, 24);
    a69 = o_shift(a69, 48);
    a54 = o_shift(a54, 72);
    a24 = o_shift(a24, 36);
    a4 = o_shift(a4, 72);
    a29 = o_neg(o_shift(a29, 12));
    { uint64_t t180 = a39; a39 = o_add(t180, a19); a19 = o_sub(t180, a19); }
    { uint64_t t181 = a49; a49 = o_add(t181, a59); a59 = o_sub(t181, a59); }
    a59 = o_shift(a59, 48);
    { uint64_t t182 = a39; a39 = o_add(t182, a49); a49 = o_sub(t182, a49); }
    { uint64_t t183 = a19; a19 = o_add(t183, a59); a59 = o_sub(t183, a59); }
    { uint64_t t184 = a64; a64 = o_add(t184, a74); a74 = o_sub(t184, a74); }
    { uint64_t t185 = a79; a79 = o_add(t185, a24); a24 = o_sub(t185, a24); }
    a24 = o_shift(a24, 48);
    { uint64_t t186 = a64; a64 = o_add(t186, a79); a79 = o_sub(t186, a79); }
    { uint64_t t187 = a74; a74 = o_add(t187, a24); a24 = o_sub(t187, a24); }
    { uint64_t t188 = a9; a9 = o_add(t188, a69); a69 = o_sub(t188, a69); }
    { uint64_t t189 = a84; a84 = o_add(t189, a4); a4 = o_sub(t189, a4); }
    a4 = o_shift(a4, 48);
    { uint64_t t190 = a9; a9 = o_add(t190, a84); a84 = o_sub(t190, a84); }
    { uint64_t t191 = a69; a69 = o_add(t191, a4); a4 = o_sub(t191, a4); }
    { uint64_t t192 = a44; a44 = o_add(t192, a54); a54 = o_sub(t192, a54); }
    { uint64_t t193 = a14; a14 = o_add(t193, a29); a29 = o_sub(t193, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t194 = a44; a44 = o_add(t194, a14); a14 = o_sub(t194, a14); }
    { uint64_t t195 = a54; a54 = o_add(t195, a29); a29 = o_sub(t195, a29); }
    { uint64_t t196 = a56; a56 = o_add(t196, a46); a46 = o_sub(t196, a46); }
    { uint64_t t197 = a71; a71 = o_add(t197, a31); a31 = o_sub(t197, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t198 = a56; a56 = o_add(t198, a71); a71 = o_sub(t198, a71); }
    { uint64_t t199 = a46; a46 = o_add(t199, a31); a31 = o_sub(t199, a31); }
    { uint64_t t200 = a81; a81 = o_add(t200, a21); a21 = o_sub(t200, a21); }
    { uint64_t t201 = a1; a1 = o_add(t201, a16); a16 = o_sub(t201, a16); }
    a16 = o_shift(a16, 48);
    { uint64_t t202 = a81; a81 = o_add(t202, a1); a1 = o_sub(t202, a1); }
    { uint64_t t203 = a21; a21 = o_add(t203, a16); a16 = o_sub(t203, a16); }
    { uint64_t t204 = a61; a61 = o_add(t204, a41); a41 = o_sub(t204, a41); }
    { uint64_t t205 = a6; a6 = o_add(t205, a11); a11 = o_sub(t205, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t206 = a61; a61 = o_add(t206, a6); a6 = o_sub(t206, a6); }
    { uint64_t t207 = a41; a41 = o_add(t207, a11); a11 = o_sub(t207, a11); }
    { uint64_t t208 = a26; a26 = o_add(t208, a76); a76 = o_sub(t208, a76); }
    { uint64_t t209 = a36; a36 = o_add(t209, a66); a66 = o_sub(t209, a66); }
    a66 = o_shift(a66, 48);
    { uint64_t t210 = a26; a26 = o_add(t210, a36); a36 = o_sub(t210, a36); }
    { uint64_t t211 = a76; a76 = o_add(t211, a66); a66 = o_sub(t211, a66); }
    a21 = o_shift(a21, 12);
    a1 = o_shift(a1, 24);
    a16 = o_shift(a16, 36);
    a41 = o_shift(a41, 24);
    a6 = o_shift(a6, 48);
    a11 = o_shift(a11, 72);
    a76 = o_shift(a76, 36);
    a36 = o_shift(a36, 72);
    a66 = o_neg(o_shift(a66, 12));
    { uint64_t t212 = a56; a56 = o_add(t212, a61); a61 = o_sub(t212, a61); }
    { uint64_t t213 = a81; a81 = o_add(t213, a26); a26 = o_sub(t213, a26); }
    a26 = o_shift(a26, 48);
    { uint64_t t214 = a56; a56 = o_add(t214, a81); a81 = o_sub(t214, a81); }
    { uint64_t t215 = a61; a61 = o_add(t215, a26); a26 = o_sub(t215, a26); }
    { uint64_t t216 = a46; a46 = o_add(t216, a41); a41 = o_sub(t216, a41); }
    { uint64_t t217 = a21; a21 = o_add(t217, a76); a76 = o_sub(t217, a76); }
    a76 = o_shift(a76, 48);
    { uint64_t t218 = a46; a46 = o_add(t218, a21); a21 = o_sub(t218, a21); }
    { uint64_t t219 = a41; a41 = o_add(t219, a76); a76 = o_sub(t219, a76); }
    { uint64_t t220 = a71; a71 = o_add(t220, a6); a6 = o_sub(t220, a6); }
    { uint64_t t221 = a1; a1 = o_add(t221, a36); a36 = o_sub(t221, a36); }
    a36 = o_shift(a36, 48);
    { uint64_t t222 = a71; a71 = o_add(t222, a1); a1 = o_sub(t222, a1); }
    { uint64_t t223 = a6; a6 = o_add(t223, a36); a36 = o_sub(t223, a36); }
    { uint64_t t224 = a31; a31 = o_add(t224, a11); a11 = o_sub(t224, a11); }
    { uint64_t t225 = a16; a16 = o_add(t225, a66); a66 = o_sub(t225, a66); }
    a66 = o_shift(a66, 48);
    { uint64_t t226 = a31; a31 = o_add(t226, a16); a16 = o_sub(t226, a16); }
    { uint64_t t227 = a11; a11 = o_add(t227, a66); a66 = o_sub(t227, a66); }
    uint64_t t228 = a51;
    a51 = o_add(a51, a56);
    a56 = o_mul(a56, 1152921504338411520ULL);
    a46 = o_mul(a46, 6259776822214049175ULL);
    a71 = o_mul(a71, 9380094172986290191ULL);
    a31 = o_mul(a31, 891943630314919127ULL);
    a61 = o_mul(a61, 17228171707553225791ULL);
    a41 = o_mul(a41, 12855743360534130886ULL);
    a6 = o_mul(a6, 6167687396920564837ULL);
    a11 = o_mul(a11, 17201834061724655524ULL);
    a81 = o_mul(a81, 15308299771656910737ULL);
    a21 = o_mul(a21, 18186005861103657533ULL);
    a1 = o_mul(a1, 53595491891823545ULL);
    a16 = o_mul(a16, 1906638201581172103ULL);
    a26 = o_mul(a26, 18303651001328874822ULL);
    a76 = o_mul(a76, 3077466521755967626ULL);
    a36 = o_mul(a36, 12423593102987598328ULL);
    a66 = o_mul(a66, 18361513053649472048ULL);
    a56 = o_add(a56, t228);
    { uint64_t t229 = a56; a56 = o_add(t229, a81); a81 = o_sub(t229, a81); }
    { uint64_t t230 = a26; a26 = o_add(t230, a61); a61 = o_sub(t230, a61); }
    a61 = o_shift(a61, 48);
    { uint64_t t231 = a56; a56 = o_add(t231, a26); a26 = o_sub(t231, a26); }
    { uint64_t t232 = a81; a81 = o_add(t232, a61); a61 = o_sub(t232, a61); }
    { uint64_t t233 = a66; a66 = o_add(t233, a11); a11 = o_sub(t233, a11); }
    { uint64_t t234 = a16; a16 = o_add(t234, a31); a31 = o_sub(t234, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t235 = a66; a66 = o_add(t235, a16); a16 = o_sub(t235, a16); }
    { uint64_t t236 = a11; a11 = o_add(t236, a31); a31 = o_sub(t236, a31); }
    { uint64_t t237 = a36; a36 = o_add(t237, a6); a6 = o_sub(t237, a6); }
    { uint64_t t238 = a1; a1 = o_add(t238, a71); a71 = o_sub(t238, a71); }
    a71 = o_shift(a71, 48);
    { uint64_t t239 = a36; a36 = o_add(t239, a1); a1 = o_sub(t239, a1); }
    { uint64_t t240 = a6; a6 = o_add(t240, a71); a71 = o_sub(t240, a71); }
    { uint64_t t241 = a76; a76 = o_add(t241, a41); a41 = o_sub(t241, a41); }
    { uint64_t t242 = a21; a21 = o_add(t242, a46); a46 = o_sub(t242, a46); }
    a46 = o_shift(a46, 48);
    { uint64_t t243 = a76; a76 = o_add(t243, a21); a21 = o_sub(t243, a21); }
    { uint64_t t244 = a41; a41 = o_add(t244, a46); a46 = o_sub(t244, a46); }
    a11 = o_shift(a11, 12);
    a16 = o_shift(a16, 24);
    a31 = o_shift(a31, 36);
    a6 = o_shift(a6, 24);
    a1 = o_shift(a1, 48);
    a71 = o_shift(a71, 72);
    a41 = o_shift(a41, 36);
    a21 = o_shift(a21, 72);
    a46 = o_neg(o_shift(a46, 12));
    { uint64_t t245 = a56; a56 = o_add(t245, a36); a36 = o_sub(t245, a36); }
    { uint64_t t246 = a66; a66 = o_add(t246, a76); a76 = o_sub(t246, a76); }
    a76 = o_shift(a76, 48);
    { uint64_t t247 = a56; a56 = o_add(t247, a66); a66 = o_sub(t247, a66); }
    { uint64_t t248 = a36; a36 = o_add(t248, a76); a76 = o_sub(t248, a76); }
    { uint64_t t249 = a81; a81 = o_add(t249, a6); a6 = o_sub(t249, a6); }
    { uint64_t t250 = a11; a11 = o_add(t250, a41); a41 = o_sub(t250, a41); }
    a41 = o_shift(a41, 48);
    { uint64_t t251 = a81; a81 = o_add(t251, a11); a11 = o_sub(t251, a11); }
    { uint64_t t252 = a6; a6 = o_add(t252, a41); a41 = o_sub(t252, a41); }
    { uint64_t t253 = a26; a26 = o_add(t253, a1); a1 = o_sub(t253, a1); }
    { uint64_t t254 = a16; a16 = o_add(t254, a21); a21 = o_sub(t254, a21); }
    a21 = o_shift(a21, 48);
    { uint64_t t255 = a26; a26 = o_add(t255, a16); a16 = o_sub(t255, a16); }
    { uint64_t t256 = a1; a1 = o_add(t256, a21); a21 = o_sub(t256, a21); }
    { uint64_t t257 = a61; a61 = o_add(t257, a71); a71 = o_sub(t257, a71); }
    { uint64_t t258 = a31; a31 = o_add(t258, a46); a46 = o_sub(t258, a46); }
    a46 = o_shift(a46, 48);
    { uint64_t t259 = a61; a61 = o_add(t259, a31); a31 = o_sub(t259, a31); }
    { uint64_t t260 = a71; a71 = o_add(t260, a46); a46 = o_sub(t260, a46); }
    { uint64_t t261 = a73; a73 = o_add(t261, a63); a63 = o_sub(t261, a63); }
    { uint64_t t262 = a3; a3 = o_add(t262, a48); a48 = o_sub(t262, a48); }
    a48 = o_shift(a48, 48);
    { uint64_t t263 = a73; a73 = o_add(t263, a3); a3 = o_sub(t263, a3); }
    { uint64_t t264 = a63; a63 = o_add(t264, a48); a48 = o_sub(t264, a48); }
    { uint64_t t265 = a13; a13 = o_add(t265, a38); a38 = o_sub(t265, a38); }
    { uint64_t t266 = a18; a18 = o_add(t266, a33); a33 = o_sub(t266, a33); }
    a33 = o_shift(a33, 48);
    { uint64_t t267 = a13; a13 = o_add(t267, a18); a18 = o_sub(t267, a18); }
    { uint64_t t268 = a38; a38 = o_add(t268, a33); a33 = o_sub(t268, a33); }
    { uint64_t t269 = a78; a78 = o_add(t269, a58); a58 = o_sub(t269, a58); }
    { uint64_t t270 = a23; a23 = o_add(t270, a28); a28 = o_sub(t270, a28); }
    a28 = o_shift(a28, 48);
    { uint64_t t271 = a78; a78 = o_add(t271, a23); a23 = o_sub(t271, a23); }
    { uint64_t t272 = a58; a58 = o_add(t272, a28); a28 = o_sub(t272, a28); }
    { uint64_t t273 = a43; a43 = o_add(t273, a8); a8 = o_sub(t273, a8); }
    { uint64_t t274 = a53; a53 = o_add(t274, a83); a83 = o_sub(t274, a83); }
    a83 = o_shift(a83, 48);
    { uint64_t t275 = a43; a43 = o_add(t275, a53); a53 = o_sub(t275, a53); }
    { uint64_t t276 = a8; a8 = o_add(t276, a83); a83 = o_sub(t276, a83); }
    a38 = o_shift(a38, 12);
    a18 = o_shift(a18, 24);
    a33 = o_shift(a33, 36);
    a58 = o_shift(a58, 24);
    a23 = o_shift(a23, 48);
    a28 = o_shift(a28, 72);
    a8 = o_shift(a8, 36);
    a53 = o_shift(a53, 72);
    a83 = o_neg(o_shift(a83, 12));
    { uint64_t t277 = a73; a73 = o_add(t277, a78); a78 = o_sub(t277, a78); }
    { uint64_t t278 = a13; a13 = o_add(t278, a43); a43 = o_sub(t278, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t279 = a73; a73 = o_add(t279, a13); a13 = o_sub(t279, a13); }
    { uint64_t t280 = a78; a78 = o_add(t280, a43); a43 = o_sub(t280, a43); }
    { uint64_t t281 = a63; a63 = o_add(t281, a58); a58 = o_sub(t281, a58); }
    { uint64_t t282 = a38; a38 = o_add(t282, a8); a8 = o_sub(t282, a8); }
    a8 = o_shift(a8, 48);
    { uint64_t t283 = a63; a63 = o_add(t283, a38); a38 = o_sub(t283, a38); }
    { uint64_t t284 = a58; a58 = o_add(t284, a8); a8 = o_sub(t284, a8); }
    { uint64_t t285 = a3; a3 = o_add(t285, a23); a23 = o_sub(t285, a23); }
    { uint64_t t286 = a18; a18 = o_add(t286, a53); a53 = o_sub(t286, a53); }
    a53 = o_shift(a53, 48);
    { uint64_t t287 = a3; a3 = o_add(t287, a18); a18 = o_sub(t287, a18); }
    { uint64_t t288 = a23; a23 = o_add(t288, a53); a53 = o_sub(t288, a53); }
    { uint64_t t289 = a48; a48 = o_add(t289, a28); a28 = o_sub(t289, a28); }
    { uint64_t t290 = a33; a33 = o_add(t290, a83); a83 = o_sub(t290, a83); }
    a83 = o_shift(a83, 48);
    { uint64_t t291 = a48; a48 = o_add(t291, a33); a33 = o_sub(t291, a33); }
    { uint64_t t292 = a28; a28 = o_add(t292, a83); a83 = o_sub(t292, a83); }
    uint64_t t293 = a68;
    a68 = o_add(a68, a73);
    a73 = o_mul(a73, 1152921504338411520ULL);
    a63 = o_mul(a63, 6259776822214049175ULL);
    a3 = o_mul(a3, 9380094172986290191ULL);
    a48 = o_mul(a48, 891943630314919127ULL);
    a78 = o_mul(a78, 17228171707553225791ULL);
    a58 = o_mul(a58, 12855743360534130886ULL);
    a23 = o_mul(a23, 6167687396920564837ULL);
    a28 = o_mul(a28, 17201834061724655524ULL);
    a13 = o_mul(a13, 15308299771656910737ULL);
    a38 = o_mul(a38, 18186005861103657533ULL);
    a18 = o_mul(a18, 53595491891823545ULL);
    a33 = o_mul(a33, 1906638201581172103ULL);
    a43 = o_mul(a43, 18303651001328874822ULL);
    a8 = o_mul(a8, 3077466521755967626ULL);
    a53 = o_mul(a53, 12423593102987598328ULL);
    a83 = o_mul(a83, 18361513053649472048ULL);
    a73 = o_add(a73, t293);
    { uint64_t t294 = a73; a73 = o_add(t294, a13); a13 = o_sub(t294, a13); }
    { uint64_t t295 = a43; a43 = o_add(t295, a78); a78 = o_sub(t295, a78); }
    a78 = o_shift(a78, 48);
    { uint64_t t296 = a73; a73 = o_add(t296, a43); a43 = o_sub(t296, a43); }
    { uint64_t t297 = a13; a13 = o_add(t297, a78); a78 = o_sub(t297, a78); }
    { uint64_t t298 = a83; a83 = o_add(t298, a28); a28 = o_sub(t298, a28); }
    { uint64_t t299 = a33; a33 = o_add(t299, a48); a48 = o_sub(t299, a48); }
    a48 = o_shift(a48, 48);
    { uint64_t t300 = a83; a83 = o_add(t300, a33); a33 = o_sub(t300, a33); }
    { uint64_t t301 = a28; a28 = o_add(t301, a48); a48 = o_sub(t301, a48); }
    { uint64_t t302 = a53; a53 = o_add(t302, a23); a23 = o_sub(t302, a23); }
    { uint64_t t303 = a18; a18 = o_add(t303, a3); a3 = o_sub(t303, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t304 = a53; a53 = o_add(t304, a18); a18 = o_sub(t304, a18); }
    { uint64_t t305 = a23; a23 = o_add(t305, a3); a3 = o_sub(t305, a3); }
    { uint64_t t306 = a8; a8 = o_add(t306, a58); a58 = o_sub(t306, a58); }
    { uint64_t t307 = a38; a38 = o_add(t307, a63); a63 = o_sub(t307, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t308 = a8; a8 = o_add(t308, a38); a38 = o_sub(t308, a38); }
    { uint64_t t309 = a58; a58 = o_add(t309, a63); a63 = o_sub(t309, a63); }
    a28 = o_shift(a28, 12);
    a33 = o_shift(a33, 24);
    a48 = o_shift(a48, 36);
    a23 = o_shift(a23, 24);
    a18 = o_shift(a18, 48);
    a3 = o_shift(a3, 72);
    a58 = o_shift(a58, 36);
    a38 = o_shift(a38, 72);
    a63 = o_neg(o_shift(a63, 12));
    { uint64_t t310 = a73; a73 = o_add(t310, a53); a53 = o_sub(t310, a53); }
    { uint64_t t311 = a83; a83 = o_add(t311, a8); a8 = o_sub(t311, a8); }
    a8 = o_shift(a8, 48);
    { uint64_t t312 = a73; a73 = o_add(t312, a83); a83 = o_sub(t312, a83); }
    { uint64_t t313 = a53; a53 = o_add(t313, a8); a8 = o_sub(t313, a8); }
    { uint64_t t314 = a13; a13 = o_add(t314, a23); a23 = o_sub(t314, a23); }
    { uint64_t t315 = a28; a28 = o_add(t315, a58); a58 = o_sub(t315, a58); }
    a58 = o_shift(a58, 48);
    { uint64_t t316 = a13; a13 = o_add(t316, a28); a28 = o_sub(t316, a28); }
    { uint64_t t317 = a23; a23 = o_add(t317, a58); a58 = o_sub(t317, a58); }
    { uint64_t t318 = a43; a43 = o_add(t318, a18); a18 = o_sub(t318, a18); }
    { uint64_t t319 = a33; a33 = o_add(t319, a38); a38 = o_sub(t319, a38); }
    a38 = o_shift(a38, 48);
    { uint64_t t320 = a43; a43 = o_add(t320, a33); a33 = o_sub(t320, a33); }
    { uint64_t t321 = a18; a18 = o_add(t321, a38); a38 = o_sub(t321, a38); }
    { uint64_t t322 = a78; a78 = o_add(t322, a3); a3 = o_sub(t322, a3); }
    { uint64_t t323 = a48; a48 = o_add(t323, a63); a63 = o_sub(t323, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t324 = a78; a78 = o_add(t324, a48); a48 = o_sub(t324, a48); }
    { uint64_t t325 = a3; a3 = o_add(t325, a63); a63 = o_sub(t325, a63); }
    { uint64_t t326 = a17; a17 = o_add(t326, a68); a68 = o_sub(t326, a68); }
    { uint64_t t327 = a51; a51 = o_add(t327, a34); a34 = o_sub(t327, a34); }
    a34 = o_shift(a34, 48);
    { uint64_t t328 = a17; a17 = o_add(t328, a51); a51 = o_sub(t328, a51); }
    { uint64_t t329 = a68; a68 = o_add(t329, a34); a34 = o_sub(t329, a34); }
    uint64_t t330 = a0;
    a0 = o_add(a0, a17);
    a17 = o_mul(a17, 4611686017353646080ULL);
    a68 = o_mul(a68, 16181989089180173841ULL);
    a51 = o_mul(a51, 5818851782451133869ULL);
    a34 = o_mul(a34, 11322249509082494407ULL);
    a17 = o_add(a17, t330);
    { uint64_t t331 = a17; a17 = o_add(t331, a51); a51 = o_sub(t331, a51); }
    { uint64_t t332 = a34; a34 = o_add(t332, a68); a68 = o_sub(t332, a68); }
    a68 = o_shift(a68, 48);
    { uint64_t t333 = a17; a17 = o_add(t333, a34); a34 = o_sub(t333, a34); }
    { uint64_t t334 = a51; a51 = o_add(t334, a68); a68 = o_sub(t334, a68); }
    { uint64_t t335 = a22; a22 = o_add(t335, a73); a73 = o_sub(t335, a73); }
    { uint64_t t336 = a56; a56 = o_add(t336, a39); a39 = o_sub(t336, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t337 = a22; a22 = o_add(t337, a56); a56 = o_sub(t337, a56); }
    { uint64_t t338 = a73; a73 = o_add(t338, a39); a39 = o_sub(t338, a39); }
    uint64_t t339 = a5;
    a5 = o_add(a5, a22);
    a22 = o_mul(a22, 4611686017353646080ULL);
    a73 = o_mul(a73, 16181989089180173841ULL);
    a56 = o_mul(a56, 5818851782451133869ULL);
    a39 = o_mul(a39, 11322249509082494407ULL);
    a22 = o_add(a22, t339);
    { uint64_t t340 = a22; a22 = o_add(t340, a56); a56 = o_sub(t340, a56); }
    { uint64_t t341 = a39; a39 = o_add(t341, a73); a73 = o_sub(t341, a73); }
    a73 = o_shift(a73, 48);
    { uint64_t t342 = a22; a22 = o_add(t342, a39); a39 = o_sub(t342, a39); }
    { uint64_t t343 = a56; a56 = o_add(t343, a73); a73 = o_sub(t343, a73); }
    { uint64_t t344 = a72; a72 = o_add(t344, a38); a38 = o_sub(t344, a38); }
    { uint64_t t345 = a21; a21 = o_add(t345, a4); a4 = o_sub(t345, a4); }
    a4 = o_shift(a4, 48);
    { uint64_t t346 = a72; a72 = o_add(t346, a21); a21 = o_sub(t346, a21); }
    { uint64_t t347 = a38; a38 = o_add(t347, a4); a4 = o_sub(t347, a4); }
    uint64_t t348 = a55;
    a55 = o_add(a55, a72);
    a72 = o_mul(a72, 4611686017353646080ULL);
    a38 = o_mul(a38, 16181989089180173841ULL);
    a21 = o_mul(a21, 5818851782451133869ULL);
    a4 = o_mul(a4, 11322249509082494407ULL);
    a72 = o_add(a72, t348);
    { uint64_t t349 = a72; a72 = o_add(t349, a21); a21 = o_sub(t349, a21); }
    { uint64_t t350 = a4; a4 = o_add(t350, a38); a38 = o_sub(t350, a38); }
    a38 = o_shift(a38, 48);
    { uint64_t t351 = a72; a72 = o_add(t351, a4); a4 = o_sub(t351, a4); }
    { uint64_t t352 = a21; a21 = o_add(t352, a38); a38 = o_sub(t352, a38); }
    { uint64_t t353 = a47; a47 = o_add(t353, a13); a13 = o_sub(t353, a13); }
    { uint64_t t354 = a81; a81 = o_add(t354, a64); a64 = o_sub(t354, a64); }
    a64 = o_shift(a64, 48);
    { uint64_t t355 = a47; a47 = o_add(t355, a81); a81 = o_sub(t355, a81); }
    { uint64_t t356 = a13; a13 = o_add(t356, a64); a64 = o_sub(t356, a64); }
    uint64_t t357 = a30;
    a30 = o_add(a30, a47);
    a47 = o_mul(a47, 4611686017353646080ULL);
    a13 = o_mul(a13, 16181989089180173841ULL);
    a81 = o_mul(a81, 5818851782451133869ULL);
    a64 = o_mul(a64, 11322249509082494407ULL);
    a47 = o_add(a47, t357);
    { uint64_t t358 = a47; a47 = o_add(t358, a81); a81 = o_sub(t358, a81); }
    { uint64_t t359 = a64; a64 = o_add(t359, a13); a13 = o_sub(t359, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t360 = a47; a47 = o_add(t360, a64); a64 = o_sub(t360, a64); }
    { uint64_t t361 = a81; a81 = o_add(t361, a13); a13 = o_sub(t361, a13); }
    { uint64_t t362 = a42; a42 = o_add(t362, a8); a8 = o_sub(t362, a8); }
    { uint64_t t363 = a76; a76 = o_add(t363, a59); a59 = o_sub(t363, a59); }
    a59 = o_shift(a59, 48);
    { uint64_t t364 = a42; a42 = o_add(t364, a76); a76 = o_sub(t364, a76); }
    { uint64_t t365 = a8; a8 = o_add(t365, a59); a59 = o_sub(t365, a59); }
    uint64_t t366 = a25;
    a25 = o_add(a25, a42);
    a42 = o_mul(a42, 4611686017353646080ULL);
    a8 = o_mul(a8, 16181989089180173841ULL);
    a76 = o_mul(a76, 5818851782451133869ULL);
    a59 = o_mul(a59, 11322249509082494407ULL);
    a42 = o_add(a42, t366);
    { uint64_t t367 = a42; a42 = o_add(t367, a76); a76 = o_sub(t367, a76); }
    { uint64_t t368 = a59; a59 = o_add(t368, a8); a8 = o_sub(t368, a8); }
    a8 = o_shift(a8, 48);
    { uint64_t t369 = a42; a42 = o_add(t369, a59); a59 = o_sub(t369, a59); }
    { uint64_t t370 = a76; a76 = o_add(t370, a8); a8 = o_sub(t370, a8); }
    { uint64_t t371 = a57; a57 = o_add(t371, a23); a23 = o_sub(t371, a23); }
    { uint64_t t372 = a6; a6 = o_add(t372, a74); a74 = o_sub(t372, a74); }
    a74 = o_shift(a74, 48);
    { uint64_t t373 = a57; a57 = o_add(t373, a6); a6 = o_sub(t373, a6); }
    { uint64_t t374 = a23; a23 = o_add(t374, a74); a74 = o_sub(t374, a74); }
    uint64_t t375 = a40;
    a40 = o_add(a40, a57);
    a57 = o_mul(a57, 4611686017353646080ULL);
    a23 = o_mul(a23, 16181989089180173841ULL);
    a6 = o_mul(a6, 5818851782451133869ULL);
    a74 = o_mul(a74, 11322249509082494407ULL);
    a57 = o_add(a57, t375);
    { uint64_t t376 = a57; a57 = o_add(t376, a6); a6 = o_sub(t376, a6); }
    { uint64_t t377 = a74; a74 = o_add(t377, a23); a23 = o_sub(t377, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t378 = a57; a57 = o_add(t378, a74); a74 = o_sub(t378, a74); }
    { uint64_t t379 = a6; a6 = o_add(t379, a23); a23 = o_sub(t379, a23); }
    { uint64_t t380 = a12; a12 = o_add(t380, a63); a63 = o_sub(t380, a63); }
    { uint64_t t381 = a46; a46 = o_add(t381, a29); a29 = o_sub(t381, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t382 = a12; a12 = o_add(t382, a46); a46 = o_sub(t382, a46); }
    { uint64_t t383 = a63; a63 = o_add(t383, a29); a29 = o_sub(t383, a29); }
    uint64_t t384 = a80;
    a80 = o_add(a80, a12);
    a12 = o_mul(a12, 4611686017353646080ULL);
    a63 = o_mul(a63, 16181989089180173841ULL);
    a46 = o_mul(a46, 5818851782451133869ULL);
    a29 = o_mul(a29, 11322249509082494407ULL);
    a12 = o_add(a12, t384);
    { uint64_t t385 = a12; a12 = o_add(t385, a46); a46 = o_sub(t385, a46); }
    { uint64_t t386 = a29; a29 = o_add(t386, a63); a63 = o_sub(t386, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t387 = a12; a12 = o_add(t387, a29); a29 = o_sub(t387, a29); }
    { uint64_t t388 = a46; a46 = o_add(t388, a63); a63 = o_sub(t388, a63); }
    { uint64_t t389 = a82; a82 = o_add(t389, a48); a48 = o_sub(t389, a48); }
    { uint64_t t390 = a31; a31 = o_add(t390, a14); a14 = o_sub(t390, a14); }
    a14 = o_shift(a14, 48);
    { uint64_t t391 = a82; a82 = o_add(t391, a31); a31 = o_sub(t391, a31); }
    { uint64_t t392 = a48; a48 = o_add(t392, a14); a14 = o_sub(t392, a14); }
    uint64_t t393 = a65;
    a65 = o_add(a65, a82);
    a82 = o_mul(a82, 4611686017353646080ULL);
    a48 = o_mul(a48, 16181989089180173841ULL);
    a31 = o_mul(a31, 5818851782451133869ULL);
    a14 = o_mul(a14, 11322249509082494407ULL);
    a82 = o_add(a82, t393);
    { uint64_t t394 = a82; a82 = o_add(t394, a31); a31 = o_sub(t394, a31); }
    { uint64_t t395 = a14; a14 = o_add(t395, a48); a48 = o_sub(t395, a48); }
    a48 = o_shift(a48, 48);
    { uint64_t t396 = a82; a82 = o_add(t396, a14); a14 = o_sub(t396, a14); }
    { uint64_t t397 = a31; a31 = o_add(t397, a48); a48 = o_sub(t397, a48); }
    { uint64_t t398 = a67; a67 = o_add(t398, a33); a33 = o_sub(t398, a33); }
    { uint64_t t399 = a16; a16 = o_add(t399, a84); a84 = o_sub(t399, a84); }
    a84 = o_shift(a84, 48);
    { uint64_t t400 = a67; a67 = o_add(t400, a16); a16 = o_sub(t400, a16); }
    { uint64_t t401 = a33; a33 = o_add(t401, a84); a84 = o_sub(t401, a84); }
    uint64_t t402 = a50;
    a50 = o_add(a50, a67);
    a67 = o_mul(a67, 4611686017353646080ULL);
    a33 = o_mul(a33, 16181989089180173841ULL);
    a16 = o_mul(a16, 5818851782451133869ULL);
    a84 = o_mul(a84, 11322249509082494407ULL);
    a67 = o_add(a67, t402);
    { uint64_t t403 = a67; a67 = o_add(t403, a16); a16 = o_sub(t403, a16); }
    { uint64_t t404 = a84; a84 = o_add(t404, a33); a33 = o_sub(t404, a33); }
    a33 = o_shift(a33, 48);
    { uint64_t t405 = a67; a67 = o_add(t405, a84); a84 = o_sub(t405, a84); }
    { uint64_t t406 = a16; a16 = o_add(t406, a33); a33 = o_sub(t406, a33); }
    { uint64_t t407 = a77; a77 = o_add(t407, a43); a43 = o_sub(t407, a43); }
    { uint64_t t408 = a26; a26 = o_add(t408, a9); a9 = o_sub(t408, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t409 = a77; a77 = o_add(t409, a26); a26 = o_sub(t409, a26); }
    { uint64_t t410 = a43; a43 = o_add(t410, a9); a9 = o_sub(t410, a9); }
    uint64_t t411 = a60;
    a60 = o_add(a60, a77);
    a77 = o_mul(a77, 4611686017353646080ULL);
    a43 = o_mul(a43, 16181989089180173841ULL);
    a26 = o_mul(a26, 5818851782451133869ULL);
    a9 = o_mul(a9, 11322249509082494407ULL);
    a77 = o_add(a77, t411);
    { uint64_t t412 = a77; a77 = o_add(t412, a26); a26 = o_sub(t412, a26); }
    { uint64_t t413 = a9; a9 = o_add(t413, a43); a43 = o_sub(t413, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t414 = a77; a77 = o_add(t414, a9); a9 = o_sub(t414, a9); }
    { uint64_t t415 = a26; a26 = o_add(t415, a43); a43 = o_sub(t415, a43); }
    { uint64_t t416 = a27; a27 = o_add(t416, a78); a78 = o_sub(t416, a78); }
    { uint64_t t417 = a61; a61 = o_add(t417, a44); a44 = o_sub(t417, a44); }
    a44 = o_shift(a44, 48);
    { uint64_t t418 = a27; a27 = o_add(t418, a61); a61 = o_sub(t418, a61); }
    { uint64_t t419 = a78; a78 = o_add(t419, a44); a44 = o_sub(t419, a44); }
    uint64_t t420 = a10;
    a10 = o_add(a10, a27);
    a27 = o_mul(a27, 4611686017353646080ULL);
    a78 = o_mul(a78, 16181989089180173841ULL);
    a61 = o_mul(a61, 5818851782451133869ULL);
    a44 = o_mul(a44, 11322249509082494407ULL);
    a27 = o_add(a27, t420);
    { uint64_t t421 = a27; a27 = o_add(t421, a61); a61 = o_sub(t421, a61); }
    { uint64_t t422 = a44; a44 = o_add(t422, a78); a78 = o_sub(t422, a78); }
    a78 = o_shift(a78, 48);
    { uint64_t t423 = a27; a27 = o_add(t423, a44); a44 = o_sub(t423, a44); }
    { uint64_t t424 = a61; a61 = o_add(t424, a78); a78 = o_sub(t424, a78); }
    { uint64_t t425 = a37; a37 = o_add(t425, a3); a3 = o_sub(t425, a3); }
    { uint64_t t426 = a71; a71 = o_add(t426, a54); a54 = o_sub(t426, a54); }
    a54 = o_shift(a54, 48);
    { uint64_t t427 = a37; a37 = o_add(t427, a71); a71 = o_sub(t427, a71); }
    { uint64_t t428 = a3; a3 = o_add(t428, a54); a54 = o_sub(t428, a54); }
    uint64_t t429 = a20;
    a20 = o_add(a20, a37);
    a37 = o_mul(a37, 4611686017353646080ULL);
    a3 = o_mul(a3, 16181989089180173841ULL);
    a71 = o_mul(a71, 5818851782451133869ULL);
    a54 = o_mul(a54, 11322249509082494407ULL);
    a37 = o_add(a37, t429);
    { uint64_t t430 = a37; a37 = o_add(t430, a71); a71 = o_sub(t430, a71); }
    { uint64_t t431 = a54; a54 = o_add(t431, a3); a3 = o_sub(t431, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t432 = a37; a37 = o_add(t432, a54); a54 = o_sub(t432, a54); }
    { uint64_t t433 = a71; a71 = o_add(t433, a3); a3 = o_sub(t433, a3); }
    { uint64_t t434 = a7; a7 = o_add(t434, a58); a58 = o_sub(t434, a58); }
    { uint64_t t435 = a41; a41 = o_add(t435, a24); a24 = o_sub(t435, a24); }
    a24 = o_shift(a24, 48);
    { uint64_t t436 = a7; a7 = o_add(t436, a41); a41 = o_sub(t436, a41); }
    { uint64_t t437 = a58; a58 = o_add(t437, a24); a24 = o_sub(t437, a24); }
    uint64_t t438 = a75;
    a75 = o_add(a75, a7);
    a7 = o_mul(a7, 4611686017353646080ULL);
    a58 = o_mul(a58, 16181989089180173841ULL);
    a41 = o_mul(a41, 5818851782451133869ULL);
    a24 = o_mul(a24, 11322249509082494407ULL);
    a7 = o_add(a7, t438);
    { uint64_t t439 = a7; a7 = o_add(t439, a41); a41 = o_sub(t439, a41); }
    { uint64_t t440 = a24; a24 = o_add(t440, a58); a58 = o_sub(t440, a58); }
    a58 = o_shift(a58, 48);
    { uint64_t t441 = a7; a7 = o_add(t441, a24); a24 = o_sub(t441, a24); }
    { uint64_t t442 = a41; a41 = o_add(t442, a58); a58 = o_sub(t442, a58); }
    { uint64_t t443 = a2; a2 = o_add(t443, a53); a53 = o_sub(t443, a53); }
    { uint64_t t444 = a36; a36 = o_add(t444, a19); a19 = o_sub(t444, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t445 = a2; a2 = o_add(t445, a36); a36 = o_sub(t445, a36); }
    { uint64_t t446 = a53; a53 = o_add(t446, a19); a19 = o_sub(t446, a19); }
    uint64_t t447 = a70;
    a70 = o_add(a70, a2);
    a2 = o_mul(a2, 4611686017353646080ULL);
    a53 = o_mul(a53, 16181989089180173841ULL);
    a36 = o_mul(a36, 5818851782451133869ULL);
    a19 = o_mul(a19, 11322249509082494407ULL);
    a2 = o_add(a2, t447);
    { uint64_t t448 = a2; a2 = o_add(t448, a36); a36 = o_sub(t448, a36); }
    { uint64_t t449 = a19; a19 = o_add(t449, a53); a53 = o_sub(t449, a53); }
    a53 = o_shift(a53, 48);
    { uint64_t t450 = a2; a2 = o_add(t450, a19); a19 = o_sub(t450, a19); }
    { uint64_t t451 = a36; a36 = o_add(t451, a53); a53 = o_sub(t451, a53); }
    { uint64_t t452 = a62; a62 = o_add(t452, a28); a28 = o_sub(t452, a28); }
    { uint64_t t453 = a11; a11 = o_add(t453, a79); a79 = o_sub(t453, a79); }
    a79 = o_shift(a79, 48);
    { uint64_t t454 = a62; a62 = o_add(t454, a11); a11 = o_sub(t454, a11); }
    { uint64_t t455 = a28; a28 = o_add(t455, a79); a79 = o_sub(t455, a79); }
    uint64_t t456 = a45;
    a45 = o_add(a45, a62);
    a62 = o_mul(a62, 4611686017353646080ULL);
    a28 = o_mul(a28, 16181989089180173841ULL);
    a11 = o_mul(a11, 5818851782451133869ULL);
    a79 = o_mul(a79, 11322249509082494407ULL);
    a62 = o_add(a62, t456);
    { uint64_t t457 = a62; a62 = o_add(t457, a11); a11 = o_sub(t457, a11); }
    { uint64_t t458 = a79; a79 = o_add(t458, a28); a28 = o_sub(t458, a28); }
    a28 = o_shift(a28, 48);
    { uint64_t t459 = a62; a62 = o_add(t459, a79); a79 = o_sub(t459, a79); }
    { uint64_t t460 = a11; a11 = o_add(t460, a28); a28 = o_sub(t460, a28); }
    { uint64_t t461 = a52; a52 = o_add(t461, a18); a18 = o_sub(t461, a18); }
    { uint64_t t462 = a1; a1 = o_add(t462, a69); a69 = o_sub(t462, a69); }
    a69 = o_shift(a69, 48);
    { uint64_t t463 = a52; a52 = o_add(t463, a1); a1 = o_sub(t463, a1); }
    { uint64_t t464 = a18; a18 = o_add(t464, a69); a69 = o_sub(t464, a69); }
    uint64_t t465 = a35;
    a35 = o_add(a35, a52);
    a52 = o_mul(a52, 4611686017353646080ULL);
    a18 = o_mul(a18, 16181989089180173841ULL);
    a1 = o_mul(a1, 5818851782451133869ULL);
    a69 = o_mul(a69, 11322249509082494407ULL);
    a52 = o_add(a52, t465);
    { uint64_t t466 = a52; a52 = o_add(t466, a1); a1 = o_sub(t466, a1); }
    { uint64_t t467 = a69; a69 = o_add(t467, a18); a18 = o_sub(t467, a18); }
    a18 = o_shift(a18, 48);
    { uint64_t t468 = a52; a52 = o_add(t468, a69); a69 = o_sub(t468, a69); }
    { uint64_t t469 = a1; a1 = o_add(t469, a18); a18 = o_sub(t469, a18); }
    { uint64_t t470 = a32; a32 = o_add(t470, a83); a83 = o_sub(t470, a83); }
    { uint64_t t471 = a66; a66 = o_add(t471, a49); a49 = o_sub(t471, a49); }
    a49 = o_shift(a49, 48);
    { uint64_t t472 = a32; a32 = o_add(t472, a66); a66 = o_sub(t472, a66); }
    { uint64_t t473 = a83; a83 = o_add(t473, a49); a49 = o_sub(t473, a49); }
    uint64_t t474 = a15;
    a15 = o_add(a15, a32);
    a32 = o_mul(a32, 4611686017353646080ULL);
    a83 = o_mul(a83, 16181989089180173841ULL);
    a66 = o_mul(a66, 5818851782451133869ULL);
    a49 = o_mul(a49, 11322249509082494407ULL);
    a32 = o_add(a32, t474);
    { uint64_t t475 = a32; a32 = o_add(t475, a66); a66 = o_sub(t475, a66); }
    { uint64_t t476 = a49; a49 = o_add(t476, a83); a83 = o_sub(t476, a83); }
    a83 = o_shift(a83, 48);
    { uint64_t t477 = a32; a32 = o_add(t477, a49); a49 = o_sub(t477, a49); }
    { uint64_t t478 = a66; a66 = o_add(t478, a83); a83 = o_sub(t478, a83); }
    v[0] = a0;
    v[1] = a22;
    v[2] = a21;
    v[3] = a13;
    v[4] = a59;
    v[5] = a40;
    v[6] = a12;
    v[7] = a31;
    v[8] = a33;
    v[9] = a9;
    v[10] = a10;
    v[11] = a37;
    v[12] = a41;
    v[13] = a53;
    v[14] = a79;
    v[15] = a35;
    v[16] = a32;
    v[17] = a51;
    v[18] = a73;
    v[19] = a4;
    v[20] = a30;
    v[21] = a42;
    v[22] = a6;
    v[23] = a63;
    v[24] = a14;
    v[25] = a50;
    v[26] = a77;
    v[27] = a61;
    v[28] = a3;
    v[29] = a24;
    v[30] = a70;
    v[31] = a62;
    v[32] = a1;
    v[33] = a83;
    v[34] = a34;
    v[35] = a5;
    v[36] = a72;
    v[37] = a81;
    v[38] = a8;
    v[39] = a74;
    v[40] = a80;
    v[41] = a82;
    v[42] = a16;
    v[43] = a43;
    v[44] = a44;
    v[45] = a20;
    v[46] = a7;
    v[47] = a36;
    v[48] = a28;
    v[49] = a69;
    v[50] = a15;
    v[51] = a17;
    v[52] = a56;
    v[53] = a38;
    v[54] = a64;
    v[55] = a25;
    v[56] = a57;
    v[57] = a46;
    v[58] = a48;
    v[59] = a84;
    v[60] = a60;
    v[61] = a27;
    v[62] = a71;
    v[63] = a58;
    v[64] = a19;
    v[65] = a45;
    v[66] = a52;
    v[67] = a66;
    v[68] = a68;
    v[69] = a39;
    v[70] = a55;
    v[71] = a47;
    v[72] = a76;
    v[73] = a23;
    v[74] = a29;
    v[75] = a65;
    v[76] = a67;
    v[77] = a26;
    v[78] = a78;
    v[79] = a54;
    v[80] = a75;
    v[81] = a2;
    v[82] = a11;
    v[83] = a18;
    v[84] = a49;
}

static void o_ntt_96(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33], a34 = v[34], a35 = v[35], a36 = v[36], a37 = v[37], a38 = v[38], a39 = v[39], a40 = v[40], a41 = v[41], a42 = v[42], a43 = v[43], a44 = v[44], a45 = v[45], a46 = v[46], a47 = v[47], a48 = v[48], a49 = v[49], a50 = v[50], a51 = v[51], a52 = v[52], a53 = v[53], a54 = v[54], a55 = v[55], a56 = v[56], a57 = v[57], a58 = v[58], a59 = v[59], a60 = v[60], a61 = v[61], a62 = v[62], a63 = v[63], a64 = v[64], a65 = v[65], a66 = v[66], a67 = v[67], a68 = v[68], a69 = v[69], a70 = v[70], a71 = v[71], a72 = v[72], a73 = v[73], a74 = v[74], a75 = v[75], a76 = v[76], a77 = v[77], a78 = v[78], a79 = v[79], a80 = v[80], a81 = v[81], a82 = v[82], a83 = v[83], a84 = v[84], a85 = v[85], a86 = v[86], a87 = v[87], a88 = v[88], a89 = v[89], a90 = v[90], a91 = v[91], a92 = v[92], a93 = v[93], a94 = v[94], a95 = v[95];
    { uint64_t t1 = a0; a0 = o_add(t1, a48); a48 = o_sub(t1, a48); }
    { uint64_t t2 = a12; a12 = o_add(t2, a60); a60 = o_sub(t2, a60); }
    { uint64_t t3 = a24; a24 = o_add(t3, a72); a72 = o_sub(t3, a72); }
    { uint64_t t4 = a36; a36 = o_add(t4, a84); a84 = o_sub(t4, a84); }
    a60 = o_shift(a60, 24);
    a72 = o_shift(a72, 48);
    a84 = o_shift(a84, 72);
    { uint64_t t5 = a0; a0 = o_add(t5, a24); a24 = o_sub(t5, a24); }
    { uint64_t t6 = a12; a12 = o_add(t6, a36); a36 = o_sub(t6, a36); }
    a36 = o_shift(a36, 48);
    { uint64_t t7 = a0; a0 = o_add(t7, a12); a12 = o_sub(t7, a12); }
    { uint64_t t8 = a24; a24 = o_add(t8, a36); a36 = o_sub(t8, a36); }
    { uint64_t t9 = a48; a48 = o_add(t9, a72); a72 = o_sub(t9, a72); }
    { uint64_t t10 = a60; a60 = o_add(t10, a84); a84 = o_sub(t10, a84); }
    a84 = o_shift(a84, 48);
    { uint64_t t11 = a48; a48 = o_add(t11, a60); a60 = o_sub(t11, a60); }
    { uint64_t t12 = a72; a72 = o_add(t12, a84); a84 = o_sub(t12, a84); }
    { uint64_t t13 = a1; a1 = o_add(t13, a49); a49 = o_sub(t13, a49); }
    { uint64_t t14 = a13; a13 = o_add(t14, a61); a61 = o_sub(t14, a61); }
    { uint64_t t15 = a25; a25 = o_add(t15, a73); a73 = o_sub(t15, a73); }
    { uint64_t t16 = a37; a37 = o_add(t16, a85); a85 = o_sub(t16, a85); }
    a61 = o_shift(a61, 24);
    a73 = o_shift(a73, 48);
    a85 = o_shift(a85, 72);
    { uint64_t t17 = a1; a1 = o_add(t17, a25); a25 = o_sub(t17, a25); }
    { uint64_t t18 = a13; a13 = o_add(t18, a37); a37 = o_sub(t18, a37); }
    a37 = o_shift(a37, 48);
    { uint64_t t19 = a1; a1 = o_add(t19, a13); a13 = o_sub(t19, a13); }
    { uint64_t t20 = a25; a25 = o_add(t20, a37); a37 = o_sub(t20, a37); }
    { uint64_t t21 = a49; a49 = o_add(t21, a73); a73 = o_sub(t21, a73); }
    { uint64_t t22 = a61; a61 = o_add(t22, a85); a85 = o_sub(t22, a85); }
    a85 = o_shift(a85, 48);
    { uint64_t t23 = a49; a49 = o_add(t23, a61); a61 = o_sub(t23, a61); }
    { uint64_t t24 = a73; a73 = o_add(t24, a85); a85 = o_sub(t24, a85); }
    { uint64_t t25 = a2; a2 = o_add(t25, a50); a50 = o_sub(t25, a50); }
    { uint64_t t26 = a14; a14 = o_add(t26, a62); a62 = o_sub(t26, a62); }
    { uint64_t t27 = a26; a26 = o_add(t27, a74); a74 = o_sub(t27, a74); }
    { uint64_t t28 = a38; a38 = o_add(t28, a86); a86 = o_sub(t28, a86); }
    a62 = o_shift(a62, 24);
    a74 = o_shift(a74, 48);
    a86 = o_shift(a86, 72);
    { uint64_t t29 = a2; a2 = o_add(t29, a26); a26 = o_sub(t29, a26); }
    { uint64_t t30 = a14; a14 = o_add(t30, a38); a38 = o_sub(t30, a38); }
    a38 = o_shift(a38, 48);
    { uint64_t t31 = a2; a2 = o_add(t31, a14); a14 = o_sub(t31, a14); }
    { uint64_t t32 = a26; a26 = o_add(t32, a38); a38 = o_sub(t32, a38); }
    { uint64_t t33 = a50; a50 = o_add(t33, a74); a74 = o_sub(t33, a74); }
    { uint64_t t34 = a62; a62 = o_add(t34, a86); a86 = o_sub(t34, a86); }
    a86 = o_shift(a86, 48);
    { uint64_t t35 = a50; a50 = o_add(t35, a62); a62 = o_sub(t35, a62); }
    { uint64_t t36 = a74; a74 = o_add(t36, a86); a86 = o_sub(t36, a86); }
    { uint64_t t37 = a3; a3 = o_add(t37, a51); a51 = o_sub(t37, a51); }
    { uint64_t t38 = a15; a15 = o_add(t38, a63); a63 = o_sub(t38, a63); }
    { uint64_t t39 = a27; a27 = o_add(t39, a75); a75 = o_sub(t39, a75); }
    { uint64_t t40 = a39; a39 = o_add(t40, a87); a87 = o_sub(t40, a87); }
    a63 = o_shift(a63, 24);
    a75 = o_shift(a75, 48);
    a87 = o_shift(a87, 72);
    { uint64_t t41 = a3; a3 = o_add(t41, a27); a27 = o_sub(t41, a27); }
    { uint64_t t42 = a15; a15 = o_add(t42, a39); a39 = o_sub(t42, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t43 = a3; a3 = o_add(t43, a15); a15 = o_sub(t43, a15); }
    { uint64_t t44 = a27; a27 = o_add(t44, a39); a39 = o_sub(t44, a39); }
    { uint64_t t45 = a51; a51 = o_add(t45, a75); a75 = o_sub(t45, a75); }
    { uint64_t t46 = a63; a63 = o_add(t46, a87); a87 = o_sub(t46, a87); }
    a87 = o_shift(a87, 48);
    { uint64_t t47 = a51; a51 = o_add(t47, a63); a63 = o_sub(t47, a63); }
    { uint64_t t48 = a75; a75 = o_add(t48, a87); a87 = o_sub(t48, a87); }
    { uint64_t t49 = a4; a4 = o_add(t49, a52); a52 = o_sub(t49, a52); }
    { uint64_t t50 = a16; a16 = o_add(t50, a64); a64 = o_sub(t50, a64); }
    { uint64_t t51 = a28; a28 = o_add(t51, a76); a76 = o_sub(t51, a76); }
    { uint64_t t52 = a40; a40 = o_add(t52, a88); a88 = o_sub(t52, a88); }
    a64 = o_shift(a64, 24);
    a76 = o_shift(a76, 48);
    a88 = o_shift(a88, 72);
    { uint64_t t53 = a4; a4 = o_add(t53, a28); a28 = o_sub(t53, a28); }
    { uint64_t t54 = a16; a16 = o_add(t54, a40); a40 = o_sub(t54, a40); }
    a40 = o_shift(a40, 48);
    { uint64_t t55 = a4; a4 = o_add(t55, a16); a16 = o_sub(t55, a16); }
    { uint64_t t56 = a28; a28 = o_add(t56, a40); a40 = o_sub(t56, a40); }
    { uint64_t t57 = a52; a52 = o_add(t57, a76); a76 = o_sub(t57, a76); }
    { uint64_t t58 = a64; a64 = o_add(t58, a88); a88 = o_sub(t58, a88); }
    a88 = o_shift(a88, 48);
    { uint64_t t59 = a52; a52 = o_add(t59, a64); a64 = o_sub(t59, a64); }
    { uint64_t t60 = a76; a76 = o_add(t60, a88); a88 = o_sub(t60, a88); }
    { uint64_t t61 = a5; a5 = o_add(t61, a53); a53 = o_sub(t61, a53); }
    { uint64_t t62 = a17; a17 = o_add(t62, a65); a65 = o_sub(t62, a65); }
    { uint64_t t63 = a29; a29 = o_add(t63, a77); a77 = o_sub(t63, a77); }
    { uint64_t t64 = a41; a41 = o_add(t64, a89); a89 = o_sub(t64, a89); }
    a65 = o_shift(a65, 24);
    a77 = o_shift(a77, 48);
    a89 = o_shift(a89, 72);
    { uint64_t t65 = a5; a5 = o_add(t65, a29); a29 = o_sub(t65, a29); }
    { uint64_t t66 = a17; a17 = o_add(t66, a41); a41 = o_sub(t66, a41); }
    a41 = o_shift(a41, 48);
    { uint64_t t67 = a5; a5 = o_add(t67, a17); a17 = o_sub(t67, a17); }
    { uint64_t t68 = a29; a29 = o_add(t68, a41); a41 = o_sub(t68, a41); }
    { uint64_t t69 = a53; a53 = o_add(t69, a77); a77 = o_sub(t69, a77); }
    { uint64_t t70 = a65; a65 = o_add(t70, a89); a89 = o_sub(t70, a89); }
    a89 = o_shift(a89, 48);
    { uint64_t t71 = a53; a53 = o_add(t71, a65); a65 = o_sub(t71, a65); }
    { uint64_t t72 = a77; a77 = o_add(t72, a89); a89 = o_sub(t72, a89); }
    { uint64_t t73 = a6; a6 = o_add(t73, a54); a54 = o_sub(t73, a54); }
    { uint64_t t74 = a18; a18 = o_add(t74, a66); a66 = o_sub(t74, a66); }
    { uint64_t t75 = a30; a30 = o_add(t75, a78); a78 = o_sub(t75, a78); }
    { uint64_t t76 = a42; a42 = o_add(t76, a90); a90 = o_sub(t76, a90); }
    a66 = o_shift(a66, 24);
    a78 = o_shift(a78, 48);
    a90 = o_shift(a90, 72);
    { uint64_t t77 = a6; a6 = o_add(t77, a30); a30 = o_sub(t77, a30); }
    { uint64_t t78 = a18; a18 = o_add(t78, a42); a42 = o_sub(t78, a42); }
    a42 = o_shift(a42, 48);
    { uint64_t t79 = a6; a6 = o_add(t79, a18); a18 = o_sub(t79, a18); }
    { uint64_t t80 = a30; a30 = o_add(t80, a42); a42 = o_sub(t80, a42); }
    { uint64_t t81 = a54; a54 = o_add(t81, a78); a78 = o_sub(t81, a78); }
    { uint64_t t82 = a66; a66 = o_add(t82, a90); a90 = o_sub(t82, a90); }
    a90 = o_shift(a90, 48);
    { uint64_t t83 = a54; a54 = o_add(t83, a66); a66 = o_sub(t83, a66); }
    { uint64_t t84 = a78; a78 = o_add(t84, a90); a90 = o_sub(t84, a90); }
    { uint64_t t85 = a7; a7 = o_add(t85, a55); a55 = o_sub(t85, a55); }
    { uint64_t t86 = a19; a19 = o_add(t86, a67); a67 = o_sub(t86, a67); }
    { uint64_t t87 = a31; a31 = o_add(t87, a79); a79 = o_sub(t87, a79); }
    { uint64_t t88 = a43; a43 = o_add(t88, a91); a91 = o_sub(t88, a91); }
    a67 = o_shift(a67, 24);
    a79 = o_shift(a79, 48);
    a91 = o_shift(a91, 72);
    { uint64_t t89 = a7; a7 = o_add(t89, a31); a31 = o_sub(t89, a31); }
    { uint64_t t90 = a19; a19 = o_add(t90, a43); a43 = o_sub(t90, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t91 = a7; a7 = o_add(t91, a19); a19 = o_sub(t91, a19); }
    { uint64_t t92 = a31; a31 = o_add(t92, a43); a43 = o_sub(t92, a43); }
    { uint64_t t93 = a55; a55 = o_add(t93, a79); a79 = o_sub(t93, a79); }
    { uint64_t t94 = a67; a67 = o_add(t94, a91); a91 = o_sub(t94, a91); }
    a91 = o_shift(a91, 48);
    { uint64_t t95 = a55; a55 = o_add(t95, a67); a67 = o_sub(t95, a67); }
    { uint64_t t96 = a79; a79 = o_add(t96, a91); a91 = o_sub(t96, a91); }
    { uint64_t t97 = a8; a8 = o_add(t97, a56); a56 = o_sub(t97, a56); }
    { uint64_t t98 = a20; a20 = o_add(t98, a68); a68 = o_sub(t98, a68); }
    { uint64_t t99 = a32; a32 = o_add(t99, a80); a80 = o_sub(t99, a80); }
    { uint64_t t100 = a44; a44 = o_add(t100, a92); a92 = o_sub(t100, a92); }
    a68 = o_shift(a68, 24);
    a80 = o_shift(a80, 48);
    a92 = o_shift(a92, 72);
    { uint64_t t101 = a8; a8 = o_add(t101, a32); a32 = o_sub(t101, a32); }
    { uint64_t t102 = a20; a20 = o_add(t102, a44); a44 = o_sub(t102, a44); }
    a44 = o_shift(a44, 48);
    { uint64_t t103 = a8; a8 = o_add(t103, a20); a20 = o_sub(t103, a20); }
    { uint64_t t104 = a32; a32 = o_add(t104, a44); a44 = o_sub(t104, a44); }
    { uint64_t t105 = a56; a56 = o_add(t105, a80); a80 = o_sub(t105, a80); }
    { uint64_t t106 = a68; a68 = o_add(t106, a92); a92 = o_sub(t106, a92); }
    a92 = o_shift(a92, 48);
    { uint64_t t107 = a56; a56 = o_add(t107, a68); a68 = o_sub(t107, a68); }
    { uint64_t t108 = a80; a80 = o_add(t108, a92); a92 = o_sub(t108, a92); }
    { uint64_t t109 = a9; a9 = o_add(t109, a57); a57 = o_sub(t109, a57); }
    { uint64_t t110 = a21; a21 = o_add(t110, a69); a69 = o_sub(t110, a69); }
    { uint64_t t111 = a33; a33 = o_add(t111, a81); a81 = o_sub(t111, a81); }
    { uint64_t t112 = a45; a45 = o_add(t112, a93); a93 = o_sub(t112, a93); }
    a69 = o_shift(a69, 24);
    a81 = o_shift(a81, 48);
    a93 = o_shift(a93, 72);
    { uint64_t t113 = a9; a9 = o_add(t113, a33); a33 = o_sub(t113, a33); }
    { uint64_t t114 = a21; a21 = o_add(t114, a45); a45 = o_sub(t114, a45); }
    a45 = o_shift(a45, 48);
    { uint64_t t115 = a9; a9 = o_add(t115, a21); a21 = o_sub(t115, a21); }
    { uint64_t t116 = a33; a33 = o_add(t116, a45); a45 = o_sub(t116, a45); }
    { uint64_t t117 = a57; a57 = o_add(t117, a81); a81 = o_sub(t117, a81); }
    { uint64_t t118 = a69; a69 = o_add(t118, a93); a93 = o_sub(t118, a93); }
    a93 = o_shift(a93, 48);
    { uint64_t t119 = a57; a57 = o_add(t119, a69); a69 = o_sub(t119, a69); }
    { uint64_t t120 = a81; a81 = o_add(t120, a93); a93 = o_sub(t120, a93); }
    { uint64_t t121 = a10; a10 = o_add(t121, a58); a58 = o_sub(t121, a58); }
    { uint64_t t122 = a22; a22 = o_add(t122, a70); a70 = o_sub(t122, a70); }
    { uint64_t t123 = a34; a34 = o_add(t123, a82); a82 = o_sub(t123, a82); }
    { uint64_t t124 = a46; a46 = o_add(t124, a94); a94 = o_sub(t124, a94); }
    a70 = o_shift(a70, 24);
    a82 = o_shift(a82, 48);
    a94 = o_shift(a94, 72);
    { uint64_t t125 = a10; a10 = o_add(t125, a34); a34 = o_sub(t125, a34); }
    { uint64_t t126 = a22; a22 = o_add(t126, a46); a46 = o_sub(t126, a46); }
    a46 = o_shift(a46, 48);
    { uint64_t t127 = a10; a10 = o_add(t127, a22); a22 = o_sub(t127, a22); }
    { uint64_t t128 = a34; a34 = o_add(t128, a46); a46 = o_sub(t128, a46); }
    { uint64_t t129 = a58; a58 = o_add(t129, a82); a82 = o_sub(t129, a82); }
    { uint64_t t130 = a70; a70 = o_add(t130, a94); a94 = o_sub(t130, a94); }
    a94 = o_shift(a94, 48);
    { uint64_t t131 = a58; a58 = o_add(t131, a70); a70 = o_sub(t131, a70); }
    { uint64_t t132 = a82; a82 = o_add(t132, a94); a94 = o_sub(t132, a94); }
    { uint64_t t133 = a11; a11 = o_add(t133, a59); a59 = o_sub(t133, a59); }
    { uint64_t t134 = a23; a23 = o_add(t134, a71); a71 = o_sub(t134, a71); }
    { uint64_t t135 = a35; a35 = o_add(t135, a83); a83 = o_sub(t135, a83); }
    { uint64_t t136 = a47; a47 = o_add(t136, a95); a95 = o_sub(t136, a95); }
    a71 = o_shift(a71, 24);
    a83 = o_shift(a83, 48);
    a95 = o_shift(a95, 72);
    { uint64_t t137 = a11; a11 = o_add(t137, a35); a35 = o_sub(t137, a35); }
    { uint64_t t138 = a23; a23 = o_add(t138, a47); a47 = o_sub(t138, a47); }
    a47 = o_shift(a47, 48);
    { uint64_t t139 = a11; a11 = o_add(t139, a23); a23 = o_sub(t139, a23); }
    { uint64_t t140 = a35; a35 = o_add(t140, a47); a47 = o_sub(t140, a47); }
    { uint64_t t141 = a59; a59 = o_add(t141, a83); a83 = o_sub(t141, a83); }
    { uint64_t t142 = a71; a71 = o_add(t142, a95); a95 = o_sub(t142, a95); }
    a95 = o_shift(a95, 48);
    { uint64_t t143 = a59; a59 = o_add(t143, a71); a71 = o_sub(t143, a71); }
    { uint64_t t144 = a83; a83 = o_add(t144, a95); a95 = o_sub(t144, a95); }
    a49 = o_shift(a49, 2);
    a25 = o_shift(a25, 4);
    a73 = o_shift(a73, 6);
    a13 = o_shift(a13, 8);
    a61 = o_shift(a61, 10);
    a37 = o_shift(a37, 12);
    a85 = o_shift(a85, 14);
    a50 = o_shift(a50, 4);
    a26 = o_shift(a26, 8);
    a74 = o_shift(a74, 12);
    a14 = o_shift(a14, 16);
    a62 = o_shift(a62, 20);
    a38 = o_shift(a38, 24);
    a86 = o_shift(a86, 28);
    a51 = o_shift(a51, 6);
    a27 = o_shift(a27, 12);
    a75 = o_shift(a75, 18);
    a15 = o_shift(a15, 24);
    a63 = o_shift(a63, 30);
    a39 = o_shift(a39, 36);
    a87 = o_shift(a87, 42);
    a52 = o_shift(a52, 8);
    a28 = o_shift(a28, 16);
    a76 = o_shift(a76, 24);
    a16 = o_shift(a16, 32);
    a64 = o_shift(a64, 40);
    a40 = o_shift(a40, 48);
    a88 = o_shift(a88, 56);
    a53 = o_shift(a53, 10);
    a29 = o_shift(a29, 20);
    a77 = o_shift(a77, 30);
    a17 = o_shift(a17, 40);
    a65 = o_shift(a65, 50);
    a41 = o_shift(a41, 60);
    a89 = o_shift(a89, 70);
    a54 = o_shift(a54, 12);
    a30 = o_shift(a30, 24);
    a78 = o_shift(a78, 36);
    a18 = o_shift(a18, 48);
    a66 = o_shift(a66, 60);
    a42 = o_shift(a42, 72);
    a90 = o_shift(a90, 84);
    a55 = o_shift(a55, 14);
    a31 = o_shift(a31, 28);
    a79 = o_shift(a79, 42);
    a19 = o_shift(a19, 56);
    a67 = o_shift(a67, 70);
    a43 = o_shift(a43, 84);
    a91 = o_neg(o_shift(a91, 2));
    a56 = o_shift(a56, 16);
    a32 = o_shift(a32, 32);
    a80 = o_shift(a80, 48);
    a20 = o_shift(a20, 64);
    a68 = o_shift(a68, 80);
    a44 = o_neg(a44);
    a92 = o_neg(o_shift(a92, 16));
    a57 = o_shift(a57, 18);
    a33 = o_shift(a33, 36);
    a81 = o_shift(a81, 54);
    a21 = o_shift(a21, 72);
    a69 = o_shift(a69, 90);
    a45 = o_neg(o_shift(a45, 12));
    a93 = o_neg(o_shift(a93, 30));
    a58 = o_shift(a58, 20);
    a34 = o_shift(a34, 40);
    a82 = o_shift(a82, 60);
    a22 = o_shift(a22, 80);
    a70 = o_neg(o_shift(a70, 4));
    a46 = o_neg(o_shift(a46, 24));
    a94 = o_neg(o_shift(a94, 44));
    a59 = o_shift(a59, 22);
    a35 = o_shift(a35, 44);
    a83 = o_shift(a83, 66);
    a23 = o_shift(a23, 88);
    a71 = o_neg(o_shift(a71, 14));
    a47 = o_neg(o_shift(a47, 36));
    a95 = o_neg(o_shift(a95, 58));
    { uint64_t t145 = a0; a0 = o_add(t145, a6); a6 = o_sub(t145, a6); }
    { uint64_t t146 = a3; a3 = o_add(t146, a9); a9 = o_sub(t146, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t147 = a0; a0 = o_add(t147, a3); a3 = o_sub(t147, a3); }
    { uint64_t t148 = a6; a6 = o_add(t148, a9); a9 = o_sub(t148, a9); }
    { uint64_t t149 = a4; a4 = o_add(t149, a10); a10 = o_sub(t149, a10); }
    { uint64_t t150 = a7; a7 = o_add(t150, a1); a1 = o_sub(t150, a1); }
    a1 = o_shift(a1, 48);
    { uint64_t t151 = a4; a4 = o_add(t151, a7); a7 = o_sub(t151, a7); }
    { uint64_t t152 = a10; a10 = o_add(t152, a1); a1 = o_sub(t152, a1); }
    { uint64_t t153 = a8; a8 = o_add(t153, a2); a2 = o_sub(t153, a2); }
    { uint64_t t154 = a11; a11 = o_add(t154, a5); a5 = o_sub(t154, a5); }
    a5 = o_shift(a5, 48);
    { uint64_t t155 = a8; a8 = o_add(t155, a11); a11 = o_sub(t155, a11); }
    { uint64_t t156 = a2; a2 = o_add(t156, a5); a5 = o_sub(t156, a5); }
    { uint64_t t157 = a0, t158 = a4, t159 = a8;
      a0 = o_add(o_add(t157, t158), t159);
      a4 = o_sub(o_add(t157, o_shift(t158, 64)), o_shift(t159, 32));
      a8 = o_add(o_sub(t157, o_shift(t158, 32)), o_shift(t159, 64)); }
    { uint64_t t160 = a6, t161 = a10, t162 = a2;
      a6 = o_add(o_add(t160, t161), t162);
      a10 = o_sub(o_add(t160, o_shift(t161, 64)), o_shift(t162, 32));
      a2 = o_add(o_sub(t160, o_shift(t161, 32)), o_shift(t162, 64)); }
    { uint64_t t163 = a3, t164 = a7, t165 = a11;
      a3 = o_add(o_add(t163, t164), t165);
      a7 = o_sub(o_add(t163, o_shift(t164, 64)), o_shift(t165, 32));
      a11 = o_add(o_sub(t163, o_shift(t164, 32)), o_shift(t165, 64)); }
    { uint64_t t166 = a9, t167 = a1, t168 = a5;
      a9 = o_add(o_add(t166, t167), t168);
      a1 = o_sub(o_add(t166, o_shift(t167, 64)), o_shift(t168, 32));
      a5 = o_add(o_sub(t166, o_shift(t167, 32)), o_shift(t168, 64)); }
    { uint64_t t169 = a48; a48 = o_add(t169, a54); a54 = o_sub(t169, a54); }
    { uint64_t t170 = a51; a51 = o_add(t170, a57); a57 = o_sub(t170, a57); }
    a57 = o_shift(a57, 48);
    { uint64_t t171 = a48; a48 = o_add(t171, a51); a51 = o_sub(t171, a51); }
    { uint64_t t172 = a54; a54 = o_add(t172, a57); a57 = o_sub(t172, a57); }
    { uint64_t t173 = a52; a52 = o_add(t173, a58); a58 = o_sub(t173, a58); }
    { uint64_t t174 = a55; a55 = o_add(t174, a49); a49 = o_sub(t174, a49); }
    a49 = o_shift(a49, 48);
    { uint64_t t175 = a52; a52 = o_add(t175, a55); a55 = o_sub(t175, a55); }
    { uint64_t t176 = a58; a58 = o_add(t176, a49); a49 = o_sub(t176, a49); }
    { uint64_t t177 = a56; a56 = o_add(t177, a50); a50 = o_sub(t177, a50); }
    { uint64_t t178 = a59; a59 = o_add(t178, a53); a53 = o_sub(t178, a53); }
    a53 = o_shift(a53, 48);
    { uint64_t t179 = a56; a56 = o_add(t179, a59); a59 = o_sub(t179, a59); }
    { uint64_t t180 = a50; a50 = o_add(t180, a53); a53 = o_sub(t180, a53); }
    { uint64_t t181 = a48, t182 = a52, t183 = a56;
      a48 = o_add(o_add(t181, t182), t183);
      a52 = o_sub(o_add(t181, o_shift(t182, 64)), o_shift(t183, 32));
      a56 = o_add(o_sub(t181, o_shift(t182, 32)), o_shift(t183, 64)); }
    { uint64_t t184 = a54, t185 = a58, t186 = a50;
      a54 = o_add(o_add(t184, t185), t186);
      a58 = o_sub(o_add(t184, o_shift(t185, 64)), o_shift(t186, 32));
      a50 = o_add(o_sub(t184, o_shift(t185, 32)), o_shift(t186, 64)); }
    { uint64_t t187 = a51, t188 = a55, t189 = a59;
      a51 = o_add(o_add(t187, t188), t189);
      a55 = o_sub(o_add(t187, o_shift(t188, 64)), o_shift(t189, 32));
      a59 = o_add(o_sub(t187, o_shift(t188, 32)), o_shift(t189, 64)); }
    { uint64_t t190 = a57, t191 = a49, t192 = a53;
      a57 = o_add(o_add(t190, t191), t192);
      a49 = o_sub(o_add(t190, o_shift(t191, 64)), o_shift(t192, 32));
      a53 = o_add(o_sub(t190, o_shift(t191, 32)), o_shift(t192, 64)); }
    { uint64_t t193 = a24; a24 = o_add(t193, a30); a30 = o_sub(t193, a30); }
    { uint64_t t194 = a27; a27 = o_add(t194, a33); a33 = o_sub(t194, a33); }
    a33 = o_shift(a33, 48);
    { uint64_t t195 = a24; a24 = o_add(t195, a27); a27 = o_sub(t195, a27); }
    { uint64_t t196 = a30; a30 = o_add(t196, a33); a33 = o_sub(t196, a33); }
    { uint64_t t197 = a28; a28 = o_add(t197, a34); a34 = o_sub(t197, a34); }
    { uint64_t t198 = a31; a31 = o_add(t198, a25); a25 = o_sub(t198, a25); }
    a25 = o_shift(a25, 48);
    { uint64_t t199 = a28; a28 = o_add(t199, a31); a31 = o_sub(t199, a31); }
    { uint64_t t200 = a34; a34 = o_add(t200, a25); a25 = o_sub(t200, a25); }
    { uint64_t t201 = a32; a32 = o_add(t201, a26); a26 = o_sub(t201, a26); }
    { uint64_t t202 = a35; a35 = o_add(t202, a29); a29 = o_sub(t202, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t203 = a32; a32 = o_add(t203, a35); a35 = o_sub(t203, a35); }
    { uint64_t t204 = a26; a26 = o_add(t204, a29); a29 = o_sub(t204, a29); }
    { uint64_t t205 = a24, t206 = a28, t207 = a32;
      a24 = o_add(o_add(t205, t206), t207);
      a28 = o_sub(o_add(t205, o_shift(t206, 64)), o_shift(t207, 32));
      a32 = o_add(o_sub(t205, o_shift(t206, 32)), o_shift(t207, 64)); }
    { uint64_t t208 = a30, t209 = a34, t210 = a26;
      a30 = o_add(o_add(t208, t209), t210);
      a34 = o_sub(o_add(t208, o_shift(t209, 64)), o_shift(t210, 32));
      a26 = o_add(o_sub(t208, o_shift(t209, 32)), o_shift(t210, 64)); }
    { uint64_t t211 = a27, t212 = a31, t213 = a35;
      a27 = o_add(o_add(t211, t212), t213);
      a31 = o_sub(o_add(t211, o_shift(t212, 64)), o_shift(t213, 32));
      a35 = o_add(o_sub(t211, o_shift(t212, 32)), o_shift(t213, 64)); }
    { uint64_t t214 = a33, t215 = a25, t216 = a29;
      a33 = o_add(o_add(t214, t215), t216);
      a25 = o_sub(o_add(t214, o_shift(t215, 64)), o_shift(t216, 32));
      a29 = o_add(o_sub(t214, o_shift(t215, 32)), o_shift(t216, 64)); }
    { uint64_t t217 = a72; a72 = o_add(t217, a78); a78 = o_sub(t217, a78); }
    { uint64_t t218 = a75; a75 = o_add(t218, a81); a81 = o_sub(t218, a81); }
    a81 = o_shift(a81, 48);
    { uint64_t t219 = a72; a72 = o_add(t219, a75); a75 = o_sub(t219, a75); }
    { uint64_t t220 = a78; a78 = o_add(t220, a81); a81 = o_sub(t220, a81); }
    { uint64_t t221 = a76; a76 = o_add(t221, a82); a82 = o_sub(t221, a82); }
    { uint64_t t222 = a79; a79 = o_add(t222, a73); a73 = o_sub(t222, a73); }
    a73 = o_shift(a73, 48);
    { uint64_t t223 = a76; a76 = o_add(t223, a79); a79 = o_sub(t223, a79); }
    { uint64_t t224 = a82; a82 = o_add(t224, a73); a73 = o_sub(t224, a73); }
    { uint64_t t225 = a80; a80 = o_add(t225, a74); a74 = o_sub(t225, a74); }
    { uint64_t t226 = a83; a83 = o_add(t226, a77); a77 = o_sub(t226, a77); }
    a77 = o_shift(a77, 48);
    { uint64_t t227 = a80; a80 = o_add(t227, a83); a83 = o_sub(t227, a83); }
    { uint64_t t228 = a74; a74 = o_add(t228, a77); a77 = o_sub(t228, a77); }
    { uint64_t t229 = a72, t230 = a76, t231 = a80;
      a72 = o_add(o_add(t229, t230), t231);
      a76 = o_sub(o_add(t229, o_shift(t230, 64)), o_shift(t231, 32));
      a80 = o_add(o_sub(t229, o_shift(t230, 32)), o_shift(t231, 64)); }
    { uint64_t t232 = a78, t233 = a82, t234 = a74;
      a78 = o_add(o_add(t232, t233), t234);
      a82 = o_sub(o_add(t232, o_shift(t233, 64)), o_shift(t234, 32));
      a74 = o_add(o_sub(t232, o_shift(t233, 32)), o_shift(t234, 64)); }
    { uint64_t t235 = a75, t236 = a79, t237 = a83;
      a75 = o_add(o_add(t235, t236), t237);
      a79 = o_sub(o_add(t235, o_shift(t236, 64)), o_shift(t237, 32));
      a83 = o_add(o_sub(t235, o_shift(t236, 32)), o_shift(t237, 64)); }
    { uint64_t t238 = a81, t239 = a73, t240 = a77;
      a81 = o_add(o_add(t238, t239), t240);
      a73 = o_sub(o_add(t238, o_shift(t239, 64)), o_shift(t240, 32));
      a77 = o_add(o_sub(t238, o_shift(t239, 32)), o_shift(t240, 64)); }
    { uint64_t t241 = a12; a12 = o_add(t241, a18); a18 = o_sub(t241, a18); }
    { uint64_t t242 = a15; a15 = o_add(t242, a21); a21 = o_sub(t242, a21); }
    a21 = o_shift(a21, 48);
    { uint64_t t243 = a12; a12 = o_add(t243, a15); a15 = o_sub(t243, a15); }
    { uint64_t t244 = a18; a18 = o_add(t244, a21); a21 = o_sub(t244, a21); }
    { uint64_t t245 = a16; a16 = o_add(t245, a22); a22 = o_sub(t245, a22); }
    { uint64_t t246 = a19; a19 = o_add(t246, a13); a13 = o_sub(t246, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t247 = a16; a16 = o_add(t247, a19); a19 = o_sub(t247, a19); }
    { uint64_t t248 = a22; a22 = o_add(t248, a13); a13 = o_sub(t248, a13); }
    { uint64_t t249 = a20; a20 = o_add(t249, a14); a14 = o_sub(t249, a14); }
    { uint64_t t250 = a23; a23 = o_add(t250, a17); a17 = o_sub(t250, a17); }
    a17 = o_shift(a17, 48);
    { uint64_t t251 = a20; a20 = o_add(t251, a23); a23 = o_sub(t251, a23); }
    { uint64_t t252 = a14; a14 = o_add(t252, a17); a17 = o_sub(t252, a17); }
    { uint64_t t253 = a12, t254 = a16, t255 = a20;
      a12 = o_add(o_add(t253, t254), t255);
      a16 = o_sub(o_add(t253, o_shift(t254, 64)), o_shift(t255, 32));
      a20 = o_add(o_sub(t253, o_shift(t254, 32)), o_shift(t255, 64)); }
    { uint64_t t256 = a18, t257 = a22, t258 = a14;
      a18 = o_add(o_add(t256, t257), t258);
      a22 = o_sub(o_add(t256, o_shift(t257, 64)), o_shift(t258, 32));
      a14 = o_add(o_sub(t256, o_shift(t257, 32)), o_shift(t258, 64)); }
    { uint64_t t259 = a15, t260 = a19, t261 = a23;
      a15 = o_add(o_add(t259, t260), t261);
      a19 = o_sub(o_add(t259, o_shift(t260, 64)), o_shift(t261, 32));
      a23 = o_add(o_sub(t259, o_shift(t260, 32)), o_shift(t261, 64)); }
    { uint64_t t262 = a21, t263 = a13, t264 = a17;
      a21 = o_add(o_add(t262, t263), t264);
      a13 = o_sub(o_add(t262, o_shift(t263, 64)), o_shift(t264, 32));
      a17 = o_add(o_sub(t262, o_shift(t263, 32)), o_shift(t264, 64)); }
    { uint64_t t265 = a60; a60 = o_add(t265, a66); a66 = o_sub(t265, a66); }
    { uint64_t t266 = a63; a63 = o_add(t266, a69); a69 = o_sub(t266, a69); }
    a69 = o_shift(a69, 48);
    { uint64_t t267 = a60; a60 = o_add(t267, a63); a63 = o_sub(t267, a63); }
    { uint64_t t268 = a66; a66 = o_add(t268, a69); a69 = o_sub(t268, a69); }
    { uint64_t t269 = a64; a64 = o_add(t269, a70); a70 = o_sub(t269, a70); }
    { uint64_t t270 = a67; a67 = o_add(t270, a61); a61 = o_sub(t270, a61); }
    a61 = o_shift(a61, 48);
    { uint64_t t271 = a64; a64 = o_add(t271, a67); a67 = o_sub(t271, a67); }
    { uint64_t t272 = a70; a70 = o_add(t272, a61); a61 = o_sub(t272, a61); }
    { uint64_t t273 = a68; a68 = o_add(t273, a62); a62 = o_sub(t273, a62); }
    { uint64_t t274 = a71; a71 = o_add(t274, a65); a65 = o_sub(t274, a65); }
    a65 = o_shift(a65, 48);
    { uint64_t t275 = a68; a68 = o_add(t275, a71); a71 = o_sub(t275, a71); }
    { uint64_t t276 = a62; a62 = o_add(t276, a65); a65 = o_sub(t276, a65); }
    { uint64_t t277 = a60, t278 = a64, t279 = a68;
      a60 = o_add(o_add(t277, t278), t279);
      a64 = o_sub(o_add(t277, o_shift(t278, 64)), o_shift(t279, 32));
      a68 = o_add(o_sub(t277, o_shift(t278, 32)), o_shift(t279, 64)); }
    { uint64_t t280 = a66, t281 = a70, t282 = a62;
      a66 = o_add(o_add(t280, t281), t282);
      a70 = o_sub(o_add(t280, o_shift(t281, 64)), o_shift(t282, 32));
      a62 = o_add(o_sub(t280, o_shift(t281, 32)), o_shift(t282, 64)); }
    { uint64_t t283 = a63, t284 = a67, t285 = a71;
      a63 = o_add(o_add(t283, t284), t285);
      a67 = o_sub(o_add(t283, o_shift(t284, 64)), o_shift(t285, 32));
      a71 = o_add(o_sub(t283, o_shift(t284, 32)), o_shift(t285, 64)); }
    { uint64_t t286 = a69, t287 = a61, t288 = a65;
      a69 = o_add(o_add(t286, t287), t288);
      a61 = o_sub(o_add(t286, o_shift(t287, 64)), o_shift(t288, 32));
      a65 = o_add(o_sub(t286, o_shift(t287, 32)), o_shift(t288, 64)); }
    { uint64_t t289 = a36; a36 = o_add(t289, a42); a42 = o_sub(t289, a42); }
    { uint64_t t290 = a39; a39 = o_add(t290, a45); a45 = o_sub(t290, a45); }
    a45 = o_shift(a45, 48);
    { uint64_t t291 = a36; a36 = o_add(t291, a39); a39 = o_sub(t291, a39); }
    { uint64_t t292 = a42; a42 = o_add(t292, a45); a45 = o_sub(t292, a45); }
    { uint64_t t293 = a40; a40 = o_add(t293, a46); a46 = o_sub(t293, a46); }
    { uint64_t t294 = a43; a43 = o_add(t294, a37); a37 = o_sub(t294, a37); }
    a37 = o_shift(a37, 48);
    { uint64_t t295 = a40; a40 = o_add(t295, a43); a43 = o_sub(t295, a43); }
    { uint64_t t296 = a46; a46 = o_add(t296, a37); a37 = o_sub(t296, a37); }
    { uint64_t t297 = a44; a44 = o_add(t297, a38); a38 = o_sub(t297, a38); }
    { uint64_t t298 = a47; a47 = o_add(t298, a41); a41 = o_sub(t298, a41); }
    a41 = o_shift(a41, 48);
    { uint64_t t299 = a44; a44 = o_add(t299, a47); a47 = o_sub(t299, a47); }
    { uint64_t t300 = a38; a38 = o_add(t300, a41); a41 = o_sub(t300, a41); }
    { uint64_t t301 = a36, t302 = a40, t303 = a44;
      a36 = o_add(o_add(t301, t302), t303);
      a40 = o_sub(o_add(t301, o_shift(t302, 64)), o_shift(t303, 32));
      a44 = o_add(o_sub(t301, o_shift(t302, 32)), o_shift(t303, 64)); }
    { uint64_t t304 = a42, t305 = a46, t306 = a38;
      a42 = o_add(o_add(t304, t305), t306);
      a46 = o_sub(o_add(t304, o_shift(t305, 64)), o_shift(t306, 32));
      a38 = o_add(o_sub(t304, o_shift(t305, 32)), o_shift(t306, 64)); }
    { uint64_t t307 = a39, t308 = a43, t309 = a47;
      a39 = o_add(o_add(t307, t308), t309);
      a43 = o_sub(o_add(t307, o_shift(t308, 64)), o_shift(t309, 32));
      a47 = o_add(o_sub(t307, o_shift(t308, 32)), o_shift(t309, 64)); }
    { uint64_t t310 = a45, t311 = a37, t312 = a41;
      a45 = o_add(o_add(t310, t311), t312);
      a37 = o_sub(o_add(t310, o_shift(t311, 64)), o_shift(t312, 32));
      a41 = o_add(o_sub(t310, o_shift(t311, 32)), o_shift(t312, 64)); }
    { uint64_t t313 = a84; a84 = o_add(t313, a90); a90 = o_sub(t313, a90); }
    { uint64_t t314 = a87; a87 = o_add(t314, a93); a93 = o_sub(t314, a93); }
    a93 = o_shift(a93, 48);
    { uint64_t t315 = a84; a84 = o_add(t315, a87); a87 = o_sub(t315, a87); }
    { uint64_t t316 = a90; a90 = o_add(t316, a93); a93 = o_sub(t316, a93); }
    { uint64_t t317 = a88; a88 = o_add(t317, a94); a94 = o_sub(t317, a94); }
    { uint64_t t318 = a91; a91 = o_add(t318, a85); a85 = o_sub(t318, a85); }
    a85 = o_shift(a85, 48);
    { uint64_t t319 = a88; a88 = o_add(t319, a91); a91 = o_sub(t319, a91); }
    { uint64_t t320 = a94; a94 = o_add(t320, a85); a85 = o_sub(t320, a85); }
    { uint64_t t321 = a92; a92 = o_add(t321, a86); a86 = o_sub(t321, a86); }
    { uint64_t t322 = a95; a95 = o_add(t322, a89); a89 = o_sub(t322, a89); }
    a89 = o_shift(a89, 48);
    { uint64_t t323 = a92; a92 = o_add(t323, a95); a95 = o_sub(t323, a95); }
    { uint64_t t324 = a86; a86 = o_add(t324, a89); a89 = o_sub(t324, a89); }
    { uint64_t t325 = a84, t326 = a88, t327 = a92;
      a84 = o_add(o_add(t325, t326), t327);
      a88 = o_sub(o_add(t325, o_shift(t326, 64)), o_shift(t327, 32));
      a92 = o_add(o_sub(t325, o_shift(t326, 32)), o_shift(t327, 64)); }
    { uint64_t t328 = a90, t329 = a94, t330 = a86;
      a90 = o_add(o_add(t328, t329), t330);
      a94 = o_sub(o_add(t328, o_shift(t329, 64)), o_shift(t330, 32));
      a86 = o_add(o_sub(t328, o_shift(t329, 32)), o_shift(t330, 64)); }
    { uint64_t t331 = a87, t332 = a91, t333 = a95;
      a87 = o_add(o_add(t331, t332), t333);
      a91 = o_sub(o_add(t331, o_shift(t332, 64)), o_shift(t333, 32));
      a95 = o_add(o_sub(t331, o_shift(t332, 32)), o_shift(t333, 64)); }
    { uint64_t t334 = a93, t335 = a85, t336 = a89;
      a93 = o_add(o_add(t334, t335), t336);
      a85 = o_sub(o_add(t334, o_shift(t335, 64)), o_shift(t336, 32));
      a89 = o_add(o_sub(t334, o_shift(t335, 32)), o_shift(t336, 64)); }
    v[0] = a0;
    v[1] = a48;
    v[2] = a24;
    v[3] = a72;
    v[4] = a12;
    v[5] = a60;
    v[6] = a36;
    v[7] = a84;
    v[8] = a10;
    v[9] = a58;
    v[10] = a34;
    v[11] = a82;
    v[12] = a22;
    v[13] = a70;
    v[14] = a46;
    v[15] = a94;
    v[16] = a11;
    v[17] = a59;
    v[18] = a35;
    v[19] = a83;
    v[20] = a23;
    v[21] = a71;
    v[22] = a47;
    v[23] = a95;
    v[24] = a9;
    v[25] = a57;
    v[26] = a33;
    v[27] = a81;
    v[28] = a21;
    v[29] = a69;
    v[30] = a45;
    v[31] = a93;
    v[32] = a4;
    v[33] = a52;
    v[34] = a28;
    v[35] = a76;
    v[36] = a16;
    v[37] = a64;
    v[38] = a40;
    v[39] = a88;
    v[40] = a2;
    v[41] = a50;
    v[42] = a26;
    v[43] = a74;
    v[44] = a14;
    v[45] = a62;
    v[46] = a38;
    v[47] = a86;
    v[48] = a3;
    v[49] = a51;
    v[50] = a27;
    v[51] = a75;
    v[52] = a15;
    v[53] = a63;
    v[54] = a39;
    v[55] = a87;
    v[56] = a1;
    v[57] = a49;
    v[58] = a25;
    v[59] = a73;
    v[60] = a13;
    v[61] = a61;
    v[62] = a37;
    v[63] = a85;
    v[64] = a8;
    v[65] = a56;
    v[66] = a32;
    v[67] = a80;
    v[68] = a20;
    v[69] = a68;
    v[70] = a44;
    v[71] = a92;
    v[72] = a6;
    v[73] = a54;
    v[74] = a30;
    v[75] = a78;
    v[76] = a18;
    v[77] = a66;
    v[78] = a42;
    v[79] = a90;
    v[80] = a7;
    v[81] = a55;
    v[82] = a31;
    v[83] = a79;
    v[84] = a19;
    v[85] = a67;
    v[86] = a43;
    v[87] = a91;
    v[88] = a5;
    v[89] = a53;
    v[90] = a29;
    v[91] = a77;
    v[92] = a17;
    v[93] = a65;
    v[94] = a41;
    v[95] = a89;
}

static void o_ntt_102(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33], a34 = v[34], a35 = v[35], a36 = v[36], a37 = v[37], a38 = v[38], a39 = v[39], a40 = v[40], a41 = v[41], a42 = v[42], a43 = v[43], a44 = v[44], a45 = v[45], a46 = v[46], a47 = v[47], a48 = v[48], a49 = v[49], a50 = v[50], a51 = v[51], a52 = v[52], a53 = v[53], a54 = v[54], a55 = v[55], a56 = v[56], a57 = v[57], a58 = v[58], a59 = v[59], a60 = v[60], a61 = v[61], a62 = v[62], a63 = v[63], a64 = v[64], a65 = v[65], a66 = v[66], a67 = v[67], a68 = v[68], a69 = v[69], a70 = v[70], a71 = v[71], a72 = v[72], a73 = v[73], a74 = v[74], a75 = v[75], a76 = v[76], a77 = v[77], a78 = v[78], a79 = v[79], a80 = v[80], a81 = v[81], a82 = v[82], a83 = v[83], a84 = v[84], a85 = v[85], a86 = v[86], a87 = v[87], a88 = v[88], a89 = v[89], a90 = v[90], a91 = v[91], a92 = v[92], a93 = v[93], a94 = v[94], a95 = v[95], a96 = v[96], a97 = v[97], a98 = v[98], a99 = v[99], a100 = v[100], a101 = v[101];
    { uint64_t t1 = a6; a6 = o_add(t1, a96); a96 = o_sub(t1, a96); }
    { uint64_t t2 = a24; a24 = o_add(t2, a78); a78 = o_sub(t2, a78); }
    a78 = o_shift(a78, 48);
    { uint64_t t3 = a6; a6 = o_add(t3, a24); a24 = o_sub(t3, a24); }
    { uint64_t t4 = a96; a96 = o_add(t4, a78); a78 = o_sub(t4, a78); }
    { uint64_t t5 = a36; a36 = o_add(t5, a66); a66 = o_sub(t5, a66); }
    { uint64_t t6 = a42; a42 = o_add(t6, a60); a60 = o_sub(t6, a60); }
    a60 = o_shift(a60, 48);
    { uint64_t t7 = a36; a36 = o_add(t7, a42); a42 = o_sub(t7, a42); }
    { uint64_t t8 = a66; a66 = o_add(t8, a60); a60 = o_sub(t8, a60); }
    { uint64_t t9 = a12; a12 = o_add(t9, a90); a90 = o_sub(t9, a90); }
    { uint64_t t10 = a48; a48 = o_add(t10, a54); a54 = o_sub(t10, a54); }
    a54 = o_shift(a54, 48);
    { uint64_t t11 = a12; a12 = o_add(t11, a48); a48 = o_sub(t11, a48); }
    { uint64_t t12 = a90; a90 = o_add(t12, a54); a54 = o_sub(t12, a54); }
    { uint64_t t13 = a72; a72 = o_add(t13, a30); a30 = o_sub(t13, a30); }
    { uint64_t t14 = a84; a84 = o_add(t14, a18); a18 = o_sub(t14, a18); }
    a18 = o_shift(a18, 48);
    { uint64_t t15 = a72; a72 = o_add(t15, a84); a84 = o_sub(t15, a84); }
    { uint64_t t16 = a30; a30 = o_add(t16, a18); a18 = o_sub(t16, a18); }
    a66 = o_shift(a66, 12);
    a42 = o_shift(a42, 24);
    a60 = o_shift(a60, 36);
    a90 = o_shift(a90, 24);
    a48 = o_shift(a48, 48);
    a54 = o_shift(a54, 72);
    a30 = o_shift(a30, 36);
    a84 = o_shift(a84, 72);
    a18 = o_neg(o_shift(a18, 12));
    { uint64_t t17 = a6; a6 = o_add(t17, a12); a12 = o_sub(t17, a12); }
    { uint64_t t18 = a36; a36 = o_add(t18, a72); a72 = o_sub(t18, a72); }
    a72 = o_shift(a72, 48);
    { uint64_t t19 = a6; a6 = o_add(t19, a36); a36 = o_sub(t19, a36); }
    { uint64_t t20 = a12; a12 = o_add(t20, a72); a72 = o_sub(t20, a72); }
    { uint64_t t21 = a96; a96 = o_add(t21, a90); a90 = o_sub(t21, a90); }
    { uint64_t t22 = a66; a66 = o_add(t22, a30); a30 = o_sub(t22, a30); }
    a30 = o_shift(a30, 48);
    { uint64_t t23 = a96; a96 = o_add(t23, a66); a66 = o_sub(t23, a66); }
    { uint64_t t24 = a90; a90 = o_add(t24, a30); a30 = o_sub(t24, a30); }
    { uint64_t t25 = a24; a24 = o_add(t25, a48); a48 = o_sub(t25, a48); }
    { uint64_t t26 = a42; a42 = o_add(t26, a84); a84 = o_sub(t26, a84); }
    a84 = o_shift(a84, 48);
    { uint64_t t27 = a24; a24 = o_add(t27, a42); a42 = o_sub(t27, a42); }
    { uint64_t t28 = a48; a48 = o_add(t28, a84); a84 = o_sub(t28, a84); }
    { uint64_t t29 = a78; a78 = o_add(t29, a54); a54 = o_sub(t29, a54); }
    { uint64_t t30 = a60; a60 = o_add(t30, a18); a18 = o_sub(t30, a18); }
    a18 = o_shift(a18, 48);
    { uint64_t t31 = a78; a78 = o_add(t31, a60); a60 = o_sub(t31, a60); }
    { uint64_t t32 = a54; a54 = o_add(t32, a18); a18 = o_sub(t32, a18); }
    uint64_t t33 = a0;
    a0 = o_add(a0, a6);
    a6 = o_mul(a6, 1152921504338411520ULL);
    a96 = o_mul(a96, 6259776822214049175ULL);
    a24 = o_mul(a24, 9380094172986290191ULL);
    a78 = o_mul(a78, 891943630314919127ULL);
    a12 = o_mul(a12, 17228171707553225791ULL);
    a90 = o_mul(a90, 12855743360534130886ULL);
    a48 = o_mul(a48, 6167687396920564837ULL);
    a54 = o_mul(a54, 17201834061724655524ULL);
    a36 = o_mul(a36, 15308299771656910737ULL);
    a66 = o_mul(a66, 18186005861103657533ULL);
    a42 = o_mul(a42, 53595491891823545ULL);
    a60 = o_mul(a60, 1906638201581172103ULL);
    a72 = o_mul(a72, 18303651001328874822ULL);
    a30 = o_mul(a30, 3077466521755967626ULL);
    a84 = o_mul(a84, 12423593102987598328ULL);
    a18 = o_mul(a18, 18361513053649472048ULL);
    a6 = o_add(a6, t33);
    { uint64_t t34 = a6; a6 = o_add(t34, a36); a36 = o_sub(t34, a36); }
    { uint64_t t35 = a72; a72 = o_add(t35, a12); a12 = o_sub(t35, a12); }
    a12 = o_shift(a12, 48);
    { uint64_t t36 = a6; a6 = o_add(t36, a72); a72 = o_sub(t36, a72); }
    { uint64_t t37 = a36; a36 = o_add(t37, a12); a12 = o_sub(t37, a12); }
    { uint64_t t38 = a18; a18 = o_add(t38, a54); a54 = o_sub(t38, a54); }
    { uint64_t t39 = a60; a60 = o_add(t39, a78); a78 = o_sub(t39, a78); }
    a78 = o_shift(a78, 48);
    { uint64_t t40 = a18; a18 = o_add(t40, a60); a60 = o_sub(t40, a60); }
    { uint64_t t41 = a54; a54 = o_add(t41, a78); a78 = o_sub(t41, a78); }
    { uint64_t t42 = a84; a84 = o_add(t42, a48); a48 = o_sub(t42, a48); }
    { uint64_t t43 = a42; a42 = o_add(t43, a24); a24 = o_sub(t43, a24); }
    a24 = o_shift(a24, 48);
    { uint64_t t44 = a84; a84 = o_add(t44, a42); a42 = o_sub(t44, a42); }
    { uint64_t t45 = a48; a48 = o_add(t45, a24); a24 = o_sub(t45, a24); }
    { uint64_t t46 = a30; a30 = o_add(t46, a90); a90 = o_sub(t46, a90); }
    { uint64_t t47 = a66; a66 = o_add(t47, a96); a96 = o_sub(t47, a96); }
    a96 = o_shift(a96, 48);
    { uint64_t t48 = a30; a30 = o_add(t48, a66); a66 = o_sub(t48, a66); }
    { uint64_t t49 = a90; a90 = o_add(t49, a96); a96 = o_sub(t49, a96); }
    a54 = o_shift(a54, 12);
    a60 = o_shift(a60, 24);
    a78 = o_shift(a78, 36);
    a48 = o_shift(a48, 24);
    a42 = o_shift(a42, 48);
    a24 = o_shift(a24, 72);
    a90 = o_shift(a90, 36);
    a66 = o_shift(a66, 72);
    a96 = o_neg(o_shift(a96, 12));
    { uint64_t t50 = a6; a6 = o_add(t50, a84); a84 = o_sub(t50, a84); }
    { uint64_t t51 = a18; a18 = o_add(t51, a30); a30 = o_sub(t51, a30); }
    a30 = o_shift(a30, 48);
    { uint64_t t52 = a6; a6 = o_add(t52, a18); a18 = o_sub(t52, a18); }
    { uint64_t t53 = a84; a84 = o_add(t53, a30); a30 = o_sub(t53, a30); }
    { uint64_t t54 = a36; a36 = o_add(t54, a48); a48 = o_sub(t54, a48); }
    { uint64_t t55 = a54; a54 = o_add(t55, a90); a90 = o_sub(t55, a90); }
    a90 = o_shift(a90, 48);
    { uint64_t t56 = a36; a36 = o_add(t56, a54); a54 = o_sub(t56, a54); }
    { uint64_t t57 = a48; a48 = o_add(t57, a90); a90 = o_sub(t57, a90); }
    { uint64_t t58 = a72; a72 = o_add(t58, a42); a42 = o_sub(t58, a42); }
    { uint64_t t59 = a60; a60 = o_add(t59, a66); a66 = o_sub(t59, a66); }
    a66 = o_shift(a66, 48);
    { uint64_t t60 = a72; a72 = o_add(t60, a60); a60 = o_sub(t60, a60); }
    { uint64_t t61 = a42; a42 = o_add(t61, a66); a66 = o_sub(t61, a66); }
    { uint64_t t62 = a12; a12 = o_add(t62, a24); a24 = o_sub(t62, a24); }
    { uint64_t t63 = a78; a78 = o_add(t63, a96); a96 = o_sub(t63, a96); }
    a96 = o_shift(a96, 48);
    { uint64_t t64 = a12; a12 = o_add(t64, a78); a78 = o_sub(t64, a78); }
    { uint64_t t65 = a24; a24 = o_add(t65, a96); a96 = o_sub(t65, a96); }
    { uint64_t t66 = a23; a23 = o_add(t66, a11); a11 = o_sub(t66, a11); }
    { uint64_t t67 = a41; a41 = o_add(t67, a95); a95 = o_sub(t67, a95); }
    a95 = o_shift(a95, 48);
    { uint64_t t68 = a23; a23 = o_add(t68, a41); a41 = o_sub(t68, a41); }
    { uint64_t t69 = a11; a11 = o_add(t69, a95); a95 = o_sub(t69, a95); }
    { uint64_t t70 = a53; a53 = o_add(t70, a83); a83 = o_sub(t70, a83); }
    { uint64_t t71 = a59; a59 = o_add(t71, a77); a77 = o_sub(t71, a77); }
    a77 = o_shift(a77, 48);
    { uint64_t t72 = a53; a53 = o_add(t72, a59); a59 = o_sub(t72, a59); }
    { uint64_t t73 = a83; a83 = o_add(t73, a77); a77 = o_sub(t73, a77); }
    { uint64_t t74 = a29; a29 = o_add(t74, a5); a5 = o_sub(t74, a5); }
    { uint64_t t75 = a65; a65 = o_add(t75, a71); a71 = o_sub(t75, a71); }
    a71 = o_shift(a71, 48);
    { uint64_t t76 = a29; a29 = o_add(t76, a65); a65 = o_sub(t76, a65); }
    { uint64_t t77 = a5; a5 = o_add(t77, a71); a71 = o_sub(t77, a71); }
    { uint64_t t78 = a89; a89 = o_add(t78, a47); a47 = o_sub(t78, a47); }
    { uint64_t t79 = a101; a101 = o_add(t79, a35); a35 = o_sub(t79, a35); }
    a35 = o_shift(a35, 48);
    { uint64_t t80 = a89; a89 = o_add(t80, a101); a101 = o_sub(t80, a101); }
    { uint64_t t81 = a47; a47 = o_add(t81, a35); a35 = o_sub(t81, a35); }
    a83 = o_shift(a83, 12);
    a59 = o_shift(a59, 24);
    a77 = o_shift(a77, 36);
    a5 = o_shift(a5, 24);
    a65 = o_shift(a65, 48);
    a71 = o_shift(a71, 72);
    a47 = o_shift(a47, 36);
    a101 = o_shift(a101, 72);
    a35 = o_neg(o_shift(a35, 12));
    { uint64_t t82 = a23; a23 = o_add(t82, a29); a29 = o_sub(t82, a29); }
    { uint64_t t83 = a53; a53 = o_add(t83, a89); a89 = o_sub(t83, a89); }
    a89 = o_shift(a89, 48);
    { uint64_t t84 = a23; a23 = o_add(t84, a53); a53 = o_sub(t84, a53); }
    { uint64_t t85 = a29; a29 = o_add(t85, a89); a89 = o_sub(t85, a89); }
    { uint64_t t86 = a11; a11 = o_add(t86, a5); a5 = o_sub(t86, a5); }
    { uint64_t t87 = a83; a83 = o_add(t87, a47); a47 = o_sub(t87, a47); }
    a47 = o_shift(a47, 48);
    { uint64_t t88 = a11; a11 = o_add(t88, a83); a83 = o_sub(t88, a83); }
    { uint64_t t89 = a5; a5 = o_add(t89, a47); a47 = o_sub(t89, a47); }
    { uint64_t t90 = a41; a41 = o_add(t90, a65); a65 = o_sub(t90, a65); }
    { uint64_t t91 = a59; a59 = o_add(t91, a101); a101 = o_sub(t91, a101); }
    a101 = o_shift(a101, 48);
    { uint64_t t92 = a41; a41 = o_add(t92, a59); a59 = o_sub(t92, a59); }
    { uint64_t t93 = a65; a65 = o_add(t93, a101); a101 = o_sub(t93, a101); }
    { uint64_t t94 = a95; a95 = o_add(t94, a71); a71 = o_sub(t94, a71); }
    { uint64_t t95 = a77; a77 = o_add(t95, a35); a35 = o_sub(t95, a35); }
    a35 = o_shift(a35, 48);
    { uint64_t t96 = a95; a95 = o_add(t96, a77); a77 = o_sub(t96, a77); }
    { uint64_t t97 = a71; a71 = o_add(t97, a35); a35 = o_sub(t97, a35); }
    uint64_t t98 = a17;
    a17 = o_add(a17, a23);
    a23 = o_mul(a23, 1152921504338411520ULL);
    a11 = o_mul(a11, 6259776822214049175ULL);
    a41 = o_mul(a41, 9380094172986290191ULL);
    a95 = o_mul(a95, 891943630314919127ULL);
    a29 = o_mul(a29, 17228171707553225791ULL);
    a5 = o_mul(a5, 12855743360534130886ULL);
    a65 = o_mul(a65, 6167687396920564837ULL);
    a71 = o_mul(a71, 17201834061724655524ULL);
    a53 = o_mul(a53, 15308299771656910737ULL);
    a83 = o_mul(a83, 18186005861103657533ULL);
    a59 = o_mul(a59, 53595491891823545ULL);
    a77 = o_mul(a77, 1906638201581172103ULL);
    a89 = o_mul(a89, 18303651001328874822ULL);
    a47 = o_mul(a47, 3077466521755967626ULL);
    a101 = o_mul(a101, 12423593102987598328ULL);
    a35 = o_mul(a35, 18361513053649472048ULL);
    a23 = o_add(a23, t98);
    { uint64_t t99 = a23; a23 = o_add(t99, a53); a53 = o_sub(t99, a53); }
    { uint64_t t100 = a89; a89 = o_add(t100, a29); a29 = o_sub(t100, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t101 = a23; a23 = o_add(t101, a89); a89 = o_sub(t101, a89); }
    { uint64_t t102 = a53; a53 = o_add(t102, a29); a29 = o_sub(t102, a29); }
    { uint64_t t103 = a35; a35 = o_add(t103, a71); a71 = o_sub(t103, a71); }
    { uint64_t t104 = a77; a77 = o_add(t104, a95); a95 = o_sub(t104, a95); }
    a95 = o_shift(a95, 48);
    { uint64_t t105 = a35; a35 = o_add(t105, a77); a77 = o_sub(t105, a77); }
    { uint64_t t106 = a71; a71 = o_add(t106, a95); a95 = o_sub(t106, a95); }
    { uint64_t t107 = a101; a101 = o_add(t107, a65); a65 = o_sub(t107, a65); }
    { uint64_t t108 = a59; a59 = o_add(t108, a41); a41 = o_sub(t108, a41); }
    a41 = o_shift(a41, 48);
    { uint64_t t109 = a101; a101 = o_add(t109, a59); a59 = o_sub(t109, a59); }
    { uint64_t t110 = a65; a65 = o_add(t110, a41); a41 = o_sub(t110, a41); }
    { uint64_t t111 = a47; a47 = o_add(t111, a5); a5 = o_sub(t111, a5); }
    { uint64_t t112 = a83; a83 = o_add(t112, a11); a11 = o_sub(t112, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t113 = a47; a47 = o_add(t113, a83); a83 = o_sub(t113, a83); }
    { uint64_t t114 = a5; a5 = o_add(t114, a11); a11 = o_sub(t114, a11); }
    a71 = o_shift(a71, 12);
    a77 = o_shift(a77, 24);
    a95 = o_shift(a95, 36);
    a65 = o_shift(a65, 24);
    a59 = o_shift(a59, 48);
    a41 = o_shift(a41, 72);
    a5 = o_shift(a5, 36);
    a83 = o_shift(a83, 72);
    a11 = o_neg(o_shift(a11, 12));
    { uint64_t t115 = a23; a23 = o_add(t115, a101); a101 = o_sub(t115, a101); }
    { uint64_t t116 = a35; a35 = o_add(t116, a47); a47 = o_sub(t116, a47); }
    a47 = o_shift(a47, 48);
    { uint64_t t117 = a23; a23 = o_add(t117, a35); a35 = o_sub(t117, a35); }
    { uint64_t t118 = a101; a101 = o_add(t118, a47); a47 = o_sub(t118, a47); }
    { uint64_t t119 = a53; a53 = o_add(t119, a65); a65 = o_sub(t119, a65); }
    { uint64_t t120 = a71; a71 = o_add(t120, a5); a5 = o_sub(t120, a5); }
    a5 = o_shift(a5, 48);
    { uint64_t t121 = a53; a53 = o_add(t121, a71); a71 = o_sub(t121, a71); }
    { uint64_t t122 = a65; a65 = o_add(t122, a5); a5 = o_sub(t122, a5); }
    { uint64_t t123 = a89; a89 = o_add(t123, a59); a59 = o_sub(t123, a59); }
    { uint64_t t124 = a77; a77 = o_add(t124, a83); a83 = o_sub(t124, a83); }
    a83 = o_shift(a83, 48);
    { uint64_t t125 = a89; a89 = o_add(t125, a77); a77 = o_sub(t125, a77); }
    { uint64_t t126 = a59; a59 = o_add(t126, a83); a83 = o_sub(t126, a83); }
    { uint64_t t127 = a29; a29 = o_add(t127, a41); a41 = o_sub(t127, a41); }
    { uint64_t t128 = a95; a95 = o_add(t128, a11); a11 = o_sub(t128, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t129 = a29; a29 = o_add(t129, a95); a95 = o_sub(t129, a95); }
    { uint64_t t130 = a41; a41 = o_add(t130, a11); a11 = o_sub(t130, a11); }
    { uint64_t t131 = a40; a40 = o_add(t131, a28); a28 = o_sub(t131, a28); }
    { uint64_t t132 = a58; a58 = o_add(t132, a10); a10 = o_sub(t132, a10); }
    a10 = o_shift(a10, 48);
    { uint64_t t133 = a40; a40 = o_add(t133, a58); a58 = o_sub(t133, a58); }
    { uint64_t t134 = a28; a28 = o_add(t134, a10); a10 = o_sub(t134, a10); }
    { uint64_t t135 = a70; a70 = o_add(t135, a100); a100 = o_sub(t135, a100); }
    { uint64_t t136 = a76; a76 = o_add(t136, a94); a94 = o_sub(t136, a94); }
    a94 = o_shift(a94, 48);
    { uint64_t t137 = a70; a70 = o_add(t137, a76); a76 = o_sub(t137, a76); }
    { uint64_t t138 = a100; a100 = o_add(t138, a94); a94 = o_sub(t138, a94); }
    { uint64_t t139 = a46; a46 = o_add(t139, a22); a22 = o_sub(t139, a22); }
    { uint64_t t140 = a82; a82 = o_add(t140, a88); a88 = o_sub(t140, a88); }
    a88 = o_shift(a88, 48);
    { uint64_t t141 = a46; a46 = o_add(t141, a82); a82 = o_sub(t141, a82); }
    { uint64_t t142 = a22; a22 = o_add(t142, a88); a88 = o_sub(t142, a88); }
    { uint64_t t143 = a4; a4 = o_add(t143, a64); a64 = o_sub(t143, a64); }
    { uint64_t t144 = a16; a16 = o_add(t144, a52); a52 = o_sub(t144, a52); }
    a52 = o_shift(a52, 48);
    { uint64_t t145 = a4; a4 = o_add(t145, a16); a16 = o_sub(t145, a16); }
    { uint64_t t146 = a64; a64 = o_add(t146, a52); a52 = o_sub(t146, a52); }
    a100 = o_shift(a100, 12);
    a76 = o_shift(a76, 24);
    a94 = o_shift(a94, 36);
    a22 = o_shift(a22, 24);
    a82 = o_shift(a82, 48);
    a88 = o_shift(a88, 72);
    a64 = o_shift(a64, 36);
    a16 = o_shift(a16, 72);
    a52 = o_neg(o_shift(a52, 12));
    { uint64_t t147 = a40; a40 = o_add(t147, a46); a46 = o_sub(t147, a46); }
    { uint64_t t148 = a70; a70 = o_add(t148, a4); a4 = o_sub(t148, a4); }
    a4 = o_shift(a4, 48);
    { uint64_t t149 = a40; a40 = o_add(t149, a70); a70 = o_sub(t149, a70); }
    { uint64_t t150 = a46; a46 = o_add(t150, a4); a4 = o_sub(t150, a4); }
    { uint64_t t151 = a28; a28 = o_add(t151, a22); a22 = o_sub(t151, a22); }
    { uint64_t t152 = a100; a100 = o_add(t152, a64); a64 = o_sub(t152, a64); }
    a64 = o_shift(a64, 48);
    { uint64_t t153 = a28; a28 = o_add(t153, a100); a100 = o_sub(t153, a100); }
    { uint64_t t154 = a22; a22 = o_add(t154, a64); a64 = o_sub(t154, a64); }
    { uint64_t t155 = a58; a58 = o_add(t155, a82); a82 = o_sub(t155, a82); }
    { uint64_t t156 = a76; a76 = o_add(t156, a16); a16 = o_sub(t156, a16); }
    a16 = o_shift(a16, 48);
    { uint64_t t157 = a58; a58 = o_add(t157, a76); a76 = o_sub(t157, a76); }
    { uint64_t t158 = a82; a82 = o_add(t158, a16); a16 = o_sub(t158, a16); }
    { uint64_t t159 = a10; a10 = o_add(t159, a88); a88 = o_sub(t159, a88); }
    { uint64_t t160 = a94; a94 = o_add(t160, a52); a52 = o_sub(t160, a52); }
    a52 = o_shift(a52, 48);
    { uint64_t t161 = a10; a10 = o_add(t161, a94); a94 = o_sub(t161, a94); }
    { uint64_t t162 = a88; a88 = o_add(t162, a52); a52 = o_sub(t162, a52); }
    uint64_t t163 = a34;
    a34 = o_add(a34, a40);
    a40 = o_mul(a40, 1152921504338411520ULL);
    a28 = o_mul(a28, 6259776822214049175ULL);
    a58 = o_mul(a58, 9380094172986290191ULL);
    a10 = o_mul(a10, 891943630314919127ULL);
    a46 = o_mul(a46, 17228171707553225791ULL);
    a22 = o_mul(a22, 12855743360534130886ULL);
    a82 = o_mul(a82, 6167687396920564837ULL);
    a88 = o_mul(a88, 17201834061724655524ULL);
    a70 = o_mul(a70, 15308299771656910737ULL);
    a100 = o_mul(a100, 18186005861103657533ULL);
    a76 = o_mul(a76, 53595491891823545ULL);
    a94 = o_mul(a94, 1906638201581172103ULL);
    a4 = o_mul(a4, 18303651001328874822ULL);
    a64 = o_mul(a64, 3077466521755967626ULL);
    a16 = o_mul(a16, 12423593102987598328ULL);
    a52 = o_mul(a52, 18361513053649472048ULL);
    a40 = o_add(a40, t163);
    { uint64_t t164 = a40; a40 = o_add(t164, a70); a70 = o_sub(t164, a70); }
    { uint64_t t165 = a4; a4 = o_add(t165, a46); a46 = o_sub(t165, a46); }
    a46 = o_shift(a46, 48);
    { uint64_t t166 = a40; a40 = o_add(t166, a4); a4 = o_sub(t166, a4); }
    { uint64_t t167 = a70; a70 = o_add(t167, a46); a46 = o_sub(t167, a46); }
    { uint64_t t168 = a52; a52 = o_add(t168, a88); a88 = o_sub(t168, a88); }
    { uint64_t t169 = a94; a94 = o_add(t169, a10); a10 = o_sub(t169, a10); }
    a10 = o_shift(a10, 48);
    { uint64_t t170 = a52; a52 = o_add(t170, a94); a94 = o_sub(t170, a94); }
    { uint64_t t171 = a88; a88 = o_add(t171, a10); a10 = o_sub(t171, a10); }
    { uint64_t t172 = a16; a16 = o_add(t172, a82); a82 = o_sub(t172, a82); }
    { uint64_t t173 = a76; a76 = o_add(t173, a58); a58 = o_sub(t173, a58); }
    a58 = o_shift(a58, 48);
    { uint64_t t174 = a16; a16 = o_add(t174, a76); a76 = o_sub(t174, a76); }
    { uint64_t t175 = a82; a82 = o_add(t175, a58); a58 = o_sub(t175, a58); }
    { uint64_t t176 = a64; a64 = o_add(t176, a22); a22 = o_sub(t176, a22); }
    { uint64_t t177 = a100; a100 = o_add(t177, a28); a28 = o_sub(t177, a28); }
    a28 = o_shift(a28, 48);
    { uint64_t t178 = a64; a64 = o_add(t178, a100); a100 = o_sub(t178, a100); }
    { uint64_t t179 = a22; a22 = o_add(t179, a28); a28 = o_sub(t179, a28); }
    a88 = o_shift(a88, 12);
    a94 = o_shift(a94, 24);
    a10 = o_shift(a10, 36);
    a82 = o_shift(a82, 24);
    a76 = o_shift(a76, 48);
    a58 = o_shift(a58, 72);
    a22 = o_shift(a22, 36);
    a100 = o_shift(a100, 72);
    a28 = o_neg(o_shift(a28, 12));
    { uint64_t t180 = a40; a40 = o_add(t180, a16); a16 = o_sub(t180, a16); }
    { uint64_t t181 = a52; a52 = o_add(t181, a64); a64 = o_sub(t181, a64); }
    a64 = o_shift(a64, 48);
    { uint64_t t182 = a40; a40 = o_add(t182, a52); a52 = o_sub(t182, a52); }
    { uint64_t t183 = a16; a16 = o_add(t183, a64); a64 = o_sub(t183, a64); }
    { uint64_t t184 = a70; a70 = o_add(t184, a82); a82 = o_sub(t184, a82); }
    { uint64_t t185 = a88; a88 = o_add(t185, a22); a22 = o_sub(t185, a22); }
    a22 = o_shift(a22, 48);
    { uint64_t t186 = a70; a70 = o_add(t186, a88); a88 = o_sub(t186, a88); }
    { uint64_t t187 = a82; a82 = o_add(t187, a22); a22 = o_sub(t187, a22); }
    { uint64_t t188 = a4; a4 = o_add(t188, a76); a76 = o_sub(t188, a76); }
    { uint64_t t189 = a94; a94 = o_add(t189, a100); a100 = o_sub(t189, a100); }
    a100 = o_shift(a100, 48);
    { uint64_t t190 = a4; a4 = o_add(t190, a94); a94 = o_sub(t190, a94); }
    { uint64_t t191 = a76; a76 = o_add(t191, a100); a100 = o_sub(t191, a100); }
    { uint64_t t192 = a46; a46 = o_add(t192, a58); a58 = o_sub(t192, a58); }
    { uint64_t t193 = a10; a10 = o_add(t193, a28); a28 = o_sub(t193, a28); }
    a28 = o_shift(a28, 48);
    { uint64_t t194 = a46; a46 = o_add(t194, a10); a10 = o_sub(t194, a10); }
    { uint64_t t195 = a58; a58 = o_add(t195, a28); a28 = o_sub(t195, a28); }
    { uint64_t t196 = a57; a57 = o_add(t196, a45); a45 = o_sub(t196, a45); }
    { uint64_t t197 = a75; a75 = o_add(t197, a27); a27 = o_sub(t197, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t198 = a57; a57 = o_add(t198, a75); a75 = o_sub(t198, a75); }
    { uint64_t t199 = a45; a45 = o_add(t199, a27); a27 = o_sub(t199, a27); }
    { uint64_t t200 = a87; a87 = o_add(t200, a15); a15 = o_sub(t200, a15); }
    { uint64_t t201 = a93; a93 = o_add(t201, a9); a9 = o_sub(t201, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t202 = a87; a87 = o_add(t202, a93); a93 = o_sub(t202, a93); }
    { uint64_t t203 = a15; a15 = o_add(t203, a9); a9 = o_sub(t203, a9); }
    { uint64_t t204 = a63; a63 = o_add(t204, a39); a39 = o_sub(t204, a39); }
    { uint64_t t205 = a99; a99 = o_add(t205, a3); a3 = o_sub(t205, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t206 = a63; a63 = o_add(t206, a99); a99 = o_sub(t206, a99); }
    { uint64_t t207 = a39; a39 = o_add(t207, a3); a3 = o_sub(t207, a3); }
    { uint64_t t208 = a21; a21 = o_add(t208, a81); a81 = o_sub(t208, a81); }
    { uint64_t t209 = a33; a33 = o_add(t209, a69); a69 = o_sub(t209, a69); }
    a69 = o_shift(a69, 48);
    { uint64_t t210 = a21; a21 = o_add(t210, a33); a33 = o_sub(t210, a33); }
    { uint64_t t211 = a81; a81 = o_add(t211, a69); a69 = o_sub(t211, a69); }
    a15 = o_shift(a15, 12);
    a93 = o_shift(a93, 24);
    a9 = o_shift(a9, 36);
    a39 = o_shift(a39, 24);
    a99 = o_shift(a99, 48);
    a3 = o_shift(a3, 72);
    a81 = o_shift(a81, 36);
    a33 = o_shift(a33, 72);
    a69 = o_neg(o_shift(a69, 12));
    { uint64_t t212 = a57; a57 = o_add(t212, a63); a63 = o_sub(t212, a63); }
    { uint64_t t213 = a87; a87 = o_add(t213, a21); a21 = o_sub(t213, a21); }
    a21 = o_shift(a21, 48);
    { uint64_t t214 = a57; a57 = o_add(t214, a87); a87 = o_sub(t214, a87); }
    { uint64_t t215 = a63; a63 = o_add(t215, a21); a21 = o_sub(t215, a21); }
    { uint64_t t216 = a45; a45 = o_add(t216, a39); a39 = o_sub(t216, a39); }
    { uint64_t t217 = a15; a15 = o_add(t217, a81); a81 = o_sub(t217, a81); }
    a81 = o_shift(a81, 48);
    { uint64_t t218 = a45; a45 = o_add(t218, a15); a15 = o_sub(t218, a15); }
    { uint64_t t219 = a39; a39 = o_add(t219, a81); a81 = o_sub(t219, a81); }
    { uint64_t t220 = a75; a75 = o_add(t220, a99); a99 = o_sub(t220, a99); }
    { uint64_t t221 = a93; a93 = o_add(t221, a33); a33 = o_sub(t221, a33); }
    a33 = o_shift(a33, 48);
    { uint64_t t222 = a75; a75 = o_add(t222, a93); a93 = o_sub(t222, a93); }
    { uint64_t t223 = a99; a99 = o_add(t223, a33); a33 = o_sub(t223, a33); }
    { uint64_t t224 = a27; a27 = o_add(t224, a3); a3 = o_sub(t224, a3); }
    { uint64_t t225 = a9; a9 = o_add(t225, a69); a69 = o_sub(t225, a69); }
    a69 = o_shift(a69, 48);
    { uint64_t t226 = a27; a27 = o_add(t226, a9); a9 = o_sub(t226, a9); }
    { uint64_t t227 = a3; a3 = o_add(t227, a69); a69 = o_sub(t227, a69); }
    uint64_t t228 = a51;
    a51 = o_add(a51, a57);
    a57 = o_mul(a57, 1152921504338411520ULL);
    a45 = o_mul(a45, 6259776822214049175ULL);
    a75 = o_mul(a75, 9380094172986290191ULL);
    a27 = o_mul(a27, 891943630314919127ULL);
    a63 = o_mul(a63, 17228171707553225791ULL);
    a39 = o_mul(a39, 12855743360534130886ULL);
    a99 = o_mul(a99, 6167687396920564837ULL);
    a3 = o_mul(a3, 17201834061724655524ULL);
    a87 = o_mul(a87, 15308299771656910737ULL);
    a15 = o_mul(a15, 18186005861103657533ULL);
    a93 = o_mul(a93, 53595491891823545ULL);
    a9 = o_mul(a9, 1906638201581172103ULL);
    a21 = o_mul(a21, 18303651001328874822ULL);
    a81 = o_mul(a81, 3077466521755967626ULL);
    a33 = o_mul(a33, 12423593102987598328ULL);
    a69 = o_mul(a69, 18361513053649472048ULL);
    a57 = o_add(a57, t228);
    { uint64_t t229 = a57; a57 = o_add(t229, a87); a87 = o_sub(t229, a87); }
    { uint64_t t230 = a21; a21 = o_add(t230, a63); a63 = o_sub(t230, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t231 = a57; a57 = o_add(t231, a21); a21 = o_sub(t231, a21); }
    { uint64_t t232 = a87; a87 = o_add(t232, a63); a63 = o_sub(t232, a63); }
    { uint64_t t233 = a69; a69 = o_add(t233, a3); a3 = o_sub(t233, a3); }
    { uint64_t t234 = a9; a9 = o_add(t234, a27); a27 = o_sub(t234, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t235 = a69; a69 = o_add(t235, a9); a9 = o_sub(t235, a9); }
    { uint64_t t236 = a3; a3 = o_add(t236, a27); a27 = o_sub(t236, a27); }
    { uint64_t t237 = a33; a33 = o_add(t237, a99); a99 = o_sub(t237, a99); }
    { uint64_t t238 = a93; a93 = o_add(t238, a75); a75 = o_sub(t238, a75); }
    a75 = o_shift(a75, 48);
    { uint64_t t239 = a33; a33 = o_add(t239, a93); a93 = o_sub(t239, a93); }
    { uint64_t t240 = a99; a99 = o_add(t240, a75); a75 = o_sub(t240, a75); }
    { uint64_t t241 = a81; a81 = o_add(t241, a39); a39 = o_sub(t241, a39); }
    { uint64_t t242 = a15; a15 = o_add(t242, a45); a45 = o_sub(t242, a45); }
    a45 = o_shift(a45, 48);
    { uint64_t t243 = a81; a81 = o_add(t243, a15); a15 = o_sub(t243, a15); }
    { uint64_t t244 = a39; a39 = o_add(t244, a45); a45 = o_sub(t244, a45); }
    a3 = o_shift(a3, 12);
    a9 = o_shift(a9, 24);
    a27 = o_shift(a27, 36);
    a99 = o_shift(a99, 24);
    a93 = o_shift(a93, 48);
    a75 = o_shift(a75, 72);
    a39 = o_shift(a39, 36);
    a15 = o_shift(a15, 72);
    a45 = o_neg(o_shift(a45, 12));
    { uint64_t t245 = a57; a57 = o_add(t245, a33); a33 = o_sub(t245, a33); }
    { uint64_t t246 = a69; a69 = o_add(t246, a81); a81 = o_sub(t246, a81); }
    a81 = o_shift(a81, 48);
    { uint64_t t247 = a57; a57 = o_add(t247, a69); a69 = o_sub(t247, a69); }
    { uint64_t t248 = a33; a33 = o_add(t248, a81); a81 = o_sub(t248, a81); }
    { uint64_t t249 = a87; a87 = o_add(t249, a99); a99 = o_sub(t249, a99); }
    { uint64_t t250 = a3; a3 = o_add(t250, a39); a39 = o_sub(t250, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t251 = a87; a87 = o_add(t251, a3); a3 = o_sub(t251, a3); }
    { uint64_t t252 = a99; a99 = o_add(t252, a39); a39 = o_sub(t252, a39); }
    { uint64_t t253 = a21; a21 = o_add(t253, a93); a93 = o_sub(t253, a93); }
    { uint64_t t254 = a9; a9 = o_add(t254, a15); a15 = o_sub(t254, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t255 = a21; a21 = o_add(t255, a9); a9 = o_sub(t255, a9); }
    { uint64_t t256 = a93; a93 = o_add(t256, a15); a15 = o_sub(t256, a15); }
    { uint64_t t257 = a63; a63 = o_add(t257, a75); a75 = o_sub(t257, a75); }
    { uint64_t t258 = a27; a27 = o_add(t258, a45); a45 = o_sub(t258, a45); }
    a45 = o_shift(a45, 48);
    { uint64_t t259 = a63; a63 = o_add(t259, a27); a27 = o_sub(t259, a27); }
    { uint64_t t260 = a75; a75 = o_add(t260, a45); a45 = o_sub(t260, a45); }
    { uint64_t t261 = a74; a74 = o_add(t261, a62); a62 = o_sub(t261, a62); }
    { uint64_t t262 = a92; a92 = o_add(t262, a44); a44 = o_sub(t262, a44); }
    a44 = o_shift(a44, 48);
    { uint64_t t263 = a74; a74 = o_add(t263, a92); a92 = o_sub(t263, a92); }
    { uint64_t t264 = a62; a62 = o_add(t264, a44); a44 = o_sub(t264, a44); }
    { uint64_t t265 = a2; a2 = o_add(t265, a32); a32 = o_sub(t265, a32); }
    { uint64_t t266 = a8; a8 = o_add(t266, a26); a26 = o_sub(t266, a26); }
    a26 = o_shift(a26, 48);
    { uint64_t t267 = a2; a2 = o_add(t267, a8); a8 = o_sub(t267, a8); }
    { uint64_t t268 = a32; a32 = o_add(t268, a26); a26 = o_sub(t268, a26); }
    { uint64_t t269 = a80; a80 = o_add(t269, a56); a56 = o_sub(t269, a56); }
    { uint64_t t270 = a14; a14 = o_add(t270, a20); a20 = o_sub(t270, a20); }
    a20 = o_shift(a20, 48);
    { uint64_t t271 = a80; a80 = o_add(t271, a14); a14 = o_sub(t271, a14); }
    { uint64_t t272 = a56; a56 = o_add(t272, a20); a20 = o_sub(t272, a20); }
    { uint64_t t273 = a38; a38 = o_add(t273, a98); a98 = o_sub(t273, a98); }
    { uint64_t t274 = a50; a50 = o_add(t274, a86); a86 = o_sub(t274, a86); }
    a86 = o_shift(a86, 48);
    { uint64_t t275 = a38; a38 = o_add(t275, a50); a50 = o_sub(t275, a50); }
    { uint64_t t276 = a98; a98 = o_add(t276, a86); a86 = o_sub(t276, a86); }
    a32 = o_shift(a32, 12);
    a8 = o_shift(a8, 24);
    a26 = o_shift(a26, 36);
    a56 = o_shift(a56, 24);
    a14 = o_shift(a14, 48);
    a20 = o_shift(a20, 72);
    a98 = o_shift(a98, 36);
    a50 = o_shift(a50, 72);
    a86 = o_neg(o_shift(a86, 12));
    { uint64_t t277 = a74; a74 = o_add(t277, a80); a80 = o_sub(t277, a80); }
    { uint64_t t278 = a2; a2 = o_add(t278, a38); a38 = o_sub(t278, a38); }
    a38 = o_shift(a38, 48);
    { uint64_t t279 = a74; a74 = o_add(t279, a2); a2 = o_sub(t279, a2); }
    { uint64_t t280 = a80; a80 = o_add(t280, a38); a38 = o_sub(t280, a38); }
    { uint64_t t281 = a62; a62 = o_add(t281, a56); a56 = o_sub(t281, a56); }
    { uint64_t t282 = a32; a32 = o_add(t282, a98); a98 = o_sub(t282, a98); }
    a98 = o_shift(a98, 48);
    { uint64_t t283 = a62; a62 = o_add(t283, a32); a32 = o_sub(t283, a32); }
    { uint64_t t284 = a56; a56 = o_add(t284, a98); a98 = o_sub(t284, a98); }
    { uint64_t t285 = a92; a92 = o_add(t285, a14); a14 = o_sub(t285, a14); }
    { uint64_t t286 = a8; a8 = o_add(t286, a50); a50 = o_sub(t286, a50); }
    a50 = o_shift(a50, 48);
    { uint64_t t287 = a92; a92 = o_add(t287, a8); a8 = o_sub(t287, a8); }
    { uint64_t t288 = a14; a14 = o_add(t288, a50); a50 = o_sub(t288, a50); }
    { uint64_t t289 = a44; a44 = o_add(t289, a20); a20 = o_sub(t289, a20); }
    { uint64_t t290 = a26; a26 = o_add(t290, a86); a86 = o_sub(t290, a86); }
    a86 = o_shift(a86, 48);
    { uint64_t t291 = a44; a44 = o_add(t291, a26); a26 = o_sub(t291, a26); }
    { uint64_t t292 = a20; a20 = o_add(t292, a86); a86 = o_sub(t292, a86); }
    uint64_t t293 = a68;
    a68 = o_add(a68, a74);
    a74 = o_mul(a74, 1152921504338411520ULL);
    a62 = o_mul(a62, 6259776822214049175ULL);
    a92 = o_mul(a92, 9380094172986290191ULL);
    a44 = o_mul(a44, 891943630314919127ULL);
    a80 = o_mul(a80, 17228171707553225791ULL);
    a56 = o_mul(a56, 12855743360534130886ULL);
    a14 = o_mul(a14, 6167687396920564837ULL);
    a20 = o_mul(a20, 17201834061724655524ULL);
    a2 = o_mul(a2, 15308299771656910737ULL);
    a32 = o_mul(a32, 18186005861103657533ULL);
    a8 = o_mul(a8, 53595491891823545ULL);
    a26 = o_mul(a26, 1906638201581172103ULL);
    a38 = o_mul(a38, 18303651001328874822ULL);
    a98 = o_mul(a98, 3077466521755967626ULL);
    a50 = o_mul(a50, 12423593102987598328ULL);
    a86 = o_mul(a86, 18361513053649472048ULL);
    a74 = o_add(a74, t293);
    { uint64_t t294 = a74; a74 = o_add(t294, a2); a2 = o_sub(t294, a2); }
    { uint64_t t295 = a38; a38 = o_add(t295, a80); a80 = o_sub(t295, a80); }
    a80 = o_shift(a80, 48);
    { uint64_t t296 = a74; a74 = o_add(t296, a38); a38 = o_sub(t296, a38); }
    { uint64_t t297 = a2; a2 = o_add(t297, a80); a80 = o_sub(t297, a80); }
    { uint64_t t298 = a86; a86 = o_add(t298, a20); a20 = o_sub(t298, a20); }
    { uint64_t t299 = a26; a26 = o_add(t299, a44); a44 = o_sub(t299, a44); }
    a44 = o_shift(a44, 48);
    { uint64_t t300 = a86; a86 = o_add(t300, a26); a26 = o_sub(t300, a26); }
    { uint64_t t301 = a20; a20 = o_add(t301, a44); a44 = o_sub(t301, a44); }
    { uint64_t t302 = a50; a50 = o_add(t302, a14); a14 = o_sub(t302, a14); }
    { uint64_t t303 = a8; a8 = o_add(t303, a92); a92 = o_sub(t303, a92); }
    a92 = o_shift(a92, 48);
    { uint64_t t304 = a50; a50 = o_add(t304, a8); a8 = o_sub(t304, a8); }
    { uint64_t t305 = a14; a14 = o_add(t305, a92); a92 = o_sub(t305, a92); }
    { uint64_t t306 = a98; a98 = o_add(t306, a56); a56 = o_sub(t306, a56); }
    { uint64_t t307 = a32; a32 = o_add(t307, a62); a62 = o_sub(t307, a62); }
    a62 = o_shift(a62, 48);
    { uint64_t t308 = a98; a98 = o_add(t308, a32); a32 = o_sub(t308, a32); }
    { uint64_t t309 = a56; a56 = o_add(t309, a62); a62 = o_sub(t309, a62); }
    a20 = o_shift(a20, 12);
    a26 = o_shift(a26, 24);
    a44 = o_shift(a44, 36);
    a14 = o_shift(a14, 24);
    a8 = o_shift(a8, 48);
    a92 = o_shift(a92, 72);
    a56 = o_shift(a56, 36);
    a32 = o_shift(a32, 72);
    a62 = o_neg(o_shift(a62, 12));
    { uint64_t t310 = a74; a74 = o_add(t310, a50); a50 = o_sub(t310, a50); }
    { uint64_t t311 = a86; a86 = o_add(t311, a98); a98 = o_sub(t311, a98); }
    a98 = o_shift(a98, 48);
    { uint64_t t312 = a74; a74 = o_add(t312, a86); a86 = o_sub(t312, a86); }
    { uint64_t t313 = a50; a50 = o_add(t313, a98); a98 = o_sub(t313, a98); }
    { uint64_t t314 = a2; a2 = o_add(t314, a14); a14 = o_sub(t314, a14); }
    { uint64_t t315 = a20; a20 = o_add(t315, a56); a56 = o_sub(t315, a56); }
    a56 = o_shift(a56, 48);
    { uint64_t t316 = a2; a2 = o_add(t316, a20); a20 = o_sub(t316, a20); }
    { uint64_t t317 = a14; a14 = o_add(t317, a56); a56 = o_sub(t317, a56); }
    { uint64_t t318 = a38; a38 = o_add(t318, a8); a8 = o_sub(t318, a8); }
    { uint64_t t319 = a26; a26 = o_add(t319, a32); a32 = o_sub(t319, a32); }
    a32 = o_shift(a32, 48);
    { uint64_t t320 = a38; a38 = o_add(t320, a26); a26 = o_sub(t320, a26); }
    { uint64_t t321 = a8; a8 = o_add(t321, a32); a32 = o_sub(t321, a32); }
    { uint64_t t322 = a80; a80 = o_add(t322, a92); a92 = o_sub(t322, a92); }
    { uint64_t t323 = a44; a44 = o_add(t323, a62); a62 = o_sub(t323, a62); }
    a62 = o_shift(a62, 48);
    { uint64_t t324 = a80; a80 = o_add(t324, a44); a44 = o_sub(t324, a44); }
    { uint64_t t325 = a92; a92 = o_add(t325, a62); a62 = o_sub(t325, a62); }
    { uint64_t t326 = a91; a91 = o_add(t326, a79); a79 = o_sub(t326, a79); }
    { uint64_t t327 = a7; a7 = o_add(t327, a61); a61 = o_sub(t327, a61); }
    a61 = o_shift(a61, 48);
    { uint64_t t328 = a91; a91 = o_add(t328, a7); a7 = o_sub(t328, a7); }
    { uint64_t t329 = a79; a79 = o_add(t329, a61); a61 = o_sub(t329, a61); }
    { uint64_t t330 = a19; a19 = o_add(t330, a49); a49 = o_sub(t330, a49); }
    { uint64_t t331 = a25; a25 = o_add(t331, a43); a43 = o_sub(t331, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t332 = a19; a19 = o_add(t332, a25); a25 = o_sub(t332, a25); }
    { uint64_t t333 = a49; a49 = o_add(t333, a43); a43 = o_sub(t333, a43); }
    { uint64_t t334 = a97; a97 = o_add(t334, a73); a73 = o_sub(t334, a73); }
    { uint64_t t335 = a31; a31 = o_add(t335, a37); a37 = o_sub(t335, a37); }
    a37 = o_shift(a37, 48);
    { uint64_t t336 = a97; a97 = o_add(t336, a31); a31 = o_sub(t336, a31); }
    { uint64_t t337 = a73; a73 = o_add(t337, a37); a37 = o_sub(t337, a37); }
    { uint64_t t338 = a55; a55 = o_add(t338, a13); a13 = o_sub(t338, a13); }
    { uint64_t t339 = a67; a67 = o_add(t339, a1); a1 = o_sub(t339, a1); }
    a1 = o_shift(a1, 48);
    { uint64_t t340 = a55; a55 = o_add(t340, a67); a67 = o_sub(t340, a67); }
    { uint64_t t341 = a13; a13 = o_add(t341, a1); a1 = o_sub(t341, a1); }
    a49 = o_shift(a49, 12);
    a25 = o_shift(a25, 24);
    a43 = o_shift(a43, 36);
    a73 = o_shift(a73, 24);
    a31 = o_shift(a31, 48);
    a37 = o_shift(a37, 72);
    a13 = o_shift(a13, 36);
    a67 = o_shift(a67, 72);
    a1 = o_neg(o_shift(a1, 12));
    { uint64_t t342 = a91; a91 = o_add(t342, a97); a97 = o_sub(t342, a97); }
    { uint64_t t343 = a19; a19 = o_add(t343, a55); a55 = o_sub(t343, a55); }
    a55 = o_shift(a55, 48);
    { uint64_t t344 = a91; a91 = o_add(t344, a19); a19 = o_sub(t344, a19); }
    { uint64_t t345 = a97; a97 = o_add(t345, a55); a55 = o_sub(t345, a55); }
    { uint64_t t346 = a79; a79 = o_add(t346, a73); a73 = o_sub(t346, a73); }
    { uint64_t t347 = a49; a49 = o_add(t347, a13); a13 = o_sub(t347, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t348 = a79; a79 = o_add(t348, a49); a49 = o_sub(t348, a49); }
    { uint64_t t349 = a73; a73 = o_add(t349, a13); a13 = o_sub(t349, a13); }
    { uint64_t t350 = a7; a7 = o_add(t350, a31); a31 = o_sub(t350, a31); }
    { uint64_t t351 = a25; a25 = o_add(t351, a67); a67 = o_sub(t351, a67); }
    a67 = o_shift(a67, 48);
    { uint64_t t352 = a7; a7 = o_add(t352, a25); a25 = o_sub(t352, a25); }
    { uint64_t t353 = a31; a31 = o_add(t353, a67); a67 = o_sub(t353, a67); }
    { uint64_t t354 = a61; a61 = o_add(t354, a37); a37 = o_sub(t354, a37); }
    { uint64_t t355 = a43; a43 = o_add(t355, a1); a1 = o_sub(t355, a1); }
    a1 = o_shift(a1, 48);
    { uint64_t t356 = a61; a61 = o_add(t356, a43); a43 = o_sub(t356, a43); }
    { uint64_t t357 = a37; a37 = o_add(t357, a1); a1 = o_sub(t357, a1); }
    uint64_t t358 = a85;
    a85 = o_add(a85, a91);
    a91 = o_mul(a91, 1152921504338411520ULL);
    a79 = o_mul(a79, 6259776822214049175ULL);
    a7 = o_mul(a7, 9380094172986290191ULL);
    a61 = o_mul(a61, 891943630314919127ULL);
    a97 = o_mul(a97, 17228171707553225791ULL);
    a73 = o_mul(a73, 12855743360534130886ULL);
    a31 = o_mul(a31, 6167687396920564837ULL);
    a37 = o_mul(a37, 17201834061724655524ULL);
    a19 = o_mul(a19, 15308299771656910737ULL);
    a49 = o_mul(a49, 18186005861103657533ULL);
    a25 = o_mul(a25, 53595491891823545ULL);
    a43 = o_mul(a43, 1906638201581172103ULL);
    a55 = o_mul(a55, 18303651001328874822ULL);
    a13 = o_mul(a13, 3077466521755967626ULL);
    a67 = o_mul(a67, 12423593102987598328ULL);
    a1 = o_mul(a1, 18361513053649472048ULL);
    a91 = o_add(a91, t358);
    { uint64_t t359 = a91; a91 = o_add(t359, a19); a19 = o_sub(t359, a19); }
    { uint64_t t360 = a55; a55 = o_add(t360, a97); a97 = o_sub(t360, a97); }
    a97 = o_shift(a97, 48);
    { uint64_t t361 = a91; a91 = o_add(t361, a55); a55 = o_sub(t361, a55); }
    { uint64_t t362 = a19; a19 = o_add(t362, a97); a97 = o_sub(t362, a97); }
    { uint64_t t363 = a1; a1 = o_add(t363, a37); a37 = o_sub(t363, a37); }
    { uint64_t t364 = a43; a43 = o_add(t364, a61); a61 = o_sub(t364, a61); }
    a61 = o_shift(a61, 48);
    { uint64_t t365 = a1; a1 = o_add(t365, a43); a43 = o_sub(t365, a43); }
    { uint64_t t366 = a37; a37 = o_add(t366, a61); a61 = o_sub(t366, a61); }
    { uint64_t t367 = a67; a67 = o_add(t367, a31); a31 = o_sub(t367, a31); }
    { uint64_t t368 = a25; a25 = o_add(t368, a7); a7 = o_sub(t368, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t369 = a67; a67 = o_add(t369, a25); a25 = o_sub(t369, a25); }
    { uint64_t t370 = a31; a31 = o_add(t370, a7); a7 = o_sub(t370, a7); }
    { uint64_t t371 = a13; a13 = o_add(t371, a73); a73 = o_sub(t371, a73); }
    { uint64_t t372 = a49; a49 = o_add(t372, a79); a79 = o_sub(t372, a79); }
    a79 = o_shift(a79, 48);
    { uint64_t t373 = a13; a13 = o_add(t373, a49); a49 = o_sub(t373, a49); }
    { uint64_t t374 = a73; a73 = o_add(t374, a79); a79 = o_sub(t374, a79); }
    a37 = o_shift(a37, 12);
    a43 = o_shift(a43, 24);
    a61 = o_shift(a61, 36);
    a31 = o_shift(a31, 24);
    a25 = o_shift(a25, 48);
    a7 = o_shift(a7, 72);
    a73 = o_shift(a73, 36);
    a49 = o_shift(a49, 72);
    a79 = o_neg(o_shift(a79, 12));
    { uint64_t t375 = a91; a91 = o_add(t375, a67); a67 = o_sub(t375, a67); }
    { uint64_t t376 = a1; a1 = o_add(t376, a13); a13 = o_sub(t376, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t377 = a91; a91 = o_add(t377, a1); a1 = o_sub(t377, a1); }
    { uint64_t t378 = a67; a67 = o_add(t378, a13); a13 = o_sub(t378, a13); }
    { uint64_t t379 = a19; a19 = o_add(t379, a31); a31 = o_sub(t379, a31); }
    { uint64_t t380 = a37; a37 = o_add(t380, a73); a73 = o_sub(t380, a73); }
    a73 = o_shift(a73, 48);
    { uint64_t t381 = a19; a19 = o_add(t381, a37); a37 = o_sub(t381, a37); }
    { uint64_t t382 = a31; a31 = o_add(t382, a73); a73 = o_sub(t382, a73); }
    { uint64_t t383 = a55; a55 = o_add(t383, a25); a25 = o_sub(t383, a25); }
    { uint64_t t384 = a43; a43 = o_add(t384, a49); a49 = o_sub(t384, a49); }
    a49 = o_shift(a49, 48);
    { uint64_t t385 = a55; a55 = o_add(t385, a43); a43 = o_sub(t385, a43); }
    { uint64_t t386 = a25; a25 = o_add(t386, a49); a49 = o_sub(t386, a49); }
    { uint64_t t387 = a97; a97 = o_add(t387, a7); a7 = o_sub(t387, a7); }
    { uint64_t t388 = a61; a61 = o_add(t388, a79); a79 = o_sub(t388, a79); }
    a79 = o_shift(a79, 48);
    { uint64_t t389 = a97; a97 = o_add(t389, a61); a61 = o_sub(t389, a61); }
    { uint64_t t390 = a7; a7 = o_add(t390, a79); a79 = o_sub(t390, a79); }
    { uint64_t t391 = a0, t392 = a34, t393 = a68;
      a0 = o_add(o_add(t391, t392), t393);
      a34 = o_sub(o_add(t391, o_shift(t392, 64)), o_shift(t393, 32));
      a68 = o_add(o_sub(t391, o_shift(t392, 32)), o_shift(t393, 64)); }
    { uint64_t t394 = a51, t395 = a85, t396 = a17;
      a51 = o_add(o_add(t394, t395), t396);
      a85 = o_sub(o_add(t394, o_shift(t395, 64)), o_shift(t396, 32));
      a17 = o_add(o_sub(t394, o_shift(t395, 32)), o_shift(t396, 64)); }
    { uint64_t t397 = a0; a0 = o_add(t397, a51); a51 = o_sub(t397, a51); }
    { uint64_t t398 = a34; a34 = o_add(t398, a85); a85 = o_sub(t398, a85); }
    { uint64_t t399 = a68; a68 = o_add(t399, a17); a17 = o_sub(t399, a17); }
    { uint64_t t400 = a6, t401 = a40, t402 = a74;
      a6 = o_add(o_add(t400, t401), t402);
      a40 = o_sub(o_add(t400, o_shift(t401, 64)), o_shift(t402, 32));
      a74 = o_add(o_sub(t400, o_shift(t401, 32)), o_shift(t402, 64)); }
    { uint64_t t403 = a57, t404 = a91, t405 = a23;
      a57 = o_add(o_add(t403, t404), t405);
      a91 = o_sub(o_add(t403, o_shift(t404, 64)), o_shift(t405, 32));
      a23 = o_add(o_sub(t403, o_shift(t404, 32)), o_shift(t405, 64)); }
    { uint64_t t406 = a6; a6 = o_add(t406, a57); a57 = o_sub(t406, a57); }
    { uint64_t t407 = a40; a40 = o_add(t407, a91); a91 = o_sub(t407, a91); }
    { uint64_t t408 = a74; a74 = o_add(t408, a23); a23 = o_sub(t408, a23); }
    { uint64_t t409 = a66, t410 = a100, t411 = a32;
      a66 = o_add(o_add(t409, t410), t411);
      a100 = o_sub(o_add(t409, o_shift(t410, 64)), o_shift(t411, 32));
      a32 = o_add(o_sub(t409, o_shift(t410, 32)), o_shift(t411, 64)); }
    { uint64_t t412 = a15, t413 = a49, t414 = a83;
      a15 = o_add(o_add(t412, t413), t414);
      a49 = o_sub(o_add(t412, o_shift(t413, 64)), o_shift(t414, 32));
      a83 = o_add(o_sub(t412, o_shift(t413, 32)), o_shift(t414, 64)); }
    { uint64_t t415 = a66; a66 = o_add(t415, a15); a15 = o_sub(t415, a15); }
    { uint64_t t416 = a100; a100 = o_add(t416, a49); a49 = o_sub(t416, a49); }
    { uint64_t t417 = a32; a32 = o_add(t417, a83); a83 = o_sub(t417, a83); }
    { uint64_t t418 = a36, t419 = a70, t420 = a2;
      a36 = o_add(o_add(t418, t419), t420);
      a70 = o_sub(o_add(t418, o_shift(t419, 64)), o_shift(t420, 32));
      a2 = o_add(o_sub(t418, o_shift(t419, 32)), o_shift(t420, 64)); }
    { uint64_t t421 = a87, t422 = a19, t423 = a53;
      a87 = o_add(o_add(t421, t422), t423);
      a19 = o_sub(o_add(t421, o_shift(t422, 64)), o_shift(t423, 32));
      a53 = o_add(o_sub(t421, o_shift(t422, 32)), o_shift(t423, 64)); }
    { uint64_t t424 = a36; a36 = o_add(t424, a87); a87 = o_sub(t424, a87); }
    { uint64_t t425 = a70; a70 = o_add(t425, a19); a19 = o_sub(t425, a19); }
    { uint64_t t426 = a2; a2 = o_add(t426, a53); a53 = o_sub(t426, a53); }
    { uint64_t t427 = a30, t428 = a64, t429 = a98;
      a30 = o_add(o_add(t427, t428), t429);
      a64 = o_sub(o_add(t427, o_shift(t428, 64)), o_shift(t429, 32));
      a98 = o_add(o_sub(t427, o_shift(t428, 32)), o_shift(t429, 64)); }
    { uint64_t t430 = a81, t431 = a13, t432 = a47;
      a81 = o_add(o_add(t430, t431), t432);
      a13 = o_sub(o_add(t430, o_shift(t431, 64)), o_shift(t432, 32));
      a47 = o_add(o_sub(t430, o_shift(t431, 32)), o_shift(t432, 64)); }
    { uint64_t t433 = a30; a30 = o_add(t433, a81); a81 = o_sub(t433, a81); }
    { uint64_t t434 = a64; a64 = o_add(t434, a13); a13 = o_sub(t434, a13); }
    { uint64_t t435 = a98; a98 = o_add(t435, a47); a47 = o_sub(t435, a47); }
    { uint64_t t436 = a48, t437 = a82, t438 = a14;
      a48 = o_add(o_add(t436, t437), t438);
      a82 = o_sub(o_add(t436, o_shift(t437, 64)), o_shift(t438, 32));
      a14 = o_add(o_sub(t436, o_shift(t437, 32)), o_shift(t438, 64)); }
    { uint64_t t439 = a99, t440 = a31, t441 = a65;
      a99 = o_add(o_add(t439, t440), t441);
      a31 = o_sub(o_add(t439, o_shift(t440, 64)), o_shift(t441, 32));
      a65 = o_add(o_sub(t439, o_shift(t440, 32)), o_shift(t441, 64)); }
    { uint64_t t442 = a48; a48 = o_add(t442, a99); a99 = o_sub(t442, a99); }
    { uint64_t t443 = a82; a82 = o_add(t443, a31); a31 = o_sub(t443, a31); }
    { uint64_t t444 = a14; a14 = o_add(t444, a65); a65 = o_sub(t444, a65); }
    { uint64_t t445 = a96, t446 = a28, t447 = a62;
      a96 = o_add(o_add(t445, t446), t447);
      a28 = o_sub(o_add(t445, o_shift(t446, 64)), o_shift(t447, 32));
      a62 = o_add(o_sub(t445, o_shift(t446, 32)), o_shift(t447, 64)); }
    { uint64_t t448 = a45, t449 = a79, t450 = a11;
      a45 = o_add(o_add(t448, t449), t450);
      a79 = o_sub(o_add(t448, o_shift(t449, 64)), o_shift(t450, 32));
      a11 = o_add(o_sub(t448, o_shift(t449, 32)), o_shift(t450, 64)); }
    { uint64_t t451 = a96; a96 = o_add(t451, a45); a45 = o_sub(t451, a45); }
    { uint64_t t452 = a28; a28 = o_add(t452, a79); a79 = o_sub(t452, a79); }
    { uint64_t t453 = a62; a62 = o_add(t453, a11); a11 = o_sub(t453, a11); }
    { uint64_t t454 = a78, t455 = a10, t456 = a44;
      a78 = o_add(o_add(t454, t455), t456);
      a10 = o_sub(o_add(t454, o_shift(t455, 64)), o_shift(t456, 32));
      a44 = o_add(o_sub(t454, o_shift(t455, 32)), o_shift(t456, 64)); }
    { uint64_t t457 = a27, t458 = a61, t459 = a95;
      a27 = o_add(o_add(t457, t458), t459);
      a61 = o_sub(o_add(t457, o_shift(t458, 64)), o_shift(t459, 32));
      a95 = o_add(o_sub(t457, o_shift(t458, 32)), o_shift(t459, 64)); }
    { uint64_t t460 = a78; a78 = o_add(t460, a27); a27 = o_sub(t460, a27); }
    { uint64_t t461 = a10; a10 = o_add(t461, a61); a61 = o_sub(t461, a61); }
    { uint64_t t462 = a44; a44 = o_add(t462, a95); a95 = o_sub(t462, a95); }
    { uint64_t t463 = a60, t464 = a94, t465 = a26;
      a60 = o_add(o_add(t463, t464), t465);
      a94 = o_sub(o_add(t463, o_shift(t464, 64)), o_shift(t465, 32));
      a26 = o_add(o_sub(t463, o_shift(t464, 32)), o_shift(t465, 64)); }
    { uint64_t t466 = a9, t467 = a43, t468 = a77;
      a9 = o_add(o_add(t466, t467), t468);
      a43 = o_sub(o_add(t466, o_shift(t467, 64)), o_shift(t468, 32));
      a77 = o_add(o_sub(t466, o_shift(t467, 32)), o_shift(t468, 64)); }
    { uint64_t t469 = a60; a60 = o_add(t469, a9); a9 = o_sub(t469, a9); }
    { uint64_t t470 = a94; a94 = o_add(t470, a43); a43 = o_sub(t470, a43); }
    { uint64_t t471 = a26; a26 = o_add(t471, a77); a77 = o_sub(t471, a77); }
    { uint64_t t472 = a72, t473 = a4, t474 = a38;
      a72 = o_add(o_add(t472, t473), t474);
      a4 = o_sub(o_add(t472, o_shift(t473, 64)), o_shift(t474, 32));
      a38 = o_add(o_sub(t472, o_shift(t473, 32)), o_shift(t474, 64)); }
    { uint64_t t475 = a21, t476 = a55, t477 = a89;
      a21 = o_add(o_add(t475, t476), t477);
      a55 = o_sub(o_add(t475, o_shift(t476, 64)), o_shift(t477, 32));
      a89 = o_add(o_sub(t475, o_shift(t476, 32)), o_shift(t477, 64)); }
    { uint64_t t478 = a72; a72 = o_add(t478, a21); a21 = o_sub(t478, a21); }
    { uint64_t t479 = a4; a4 = o_add(t479, a55); a55 = o_sub(t479, a55); }
    { uint64_t t480 = a38; a38 = o_add(t480, a89); a89 = o_sub(t480, a89); }
    { uint64_t t481 = a12, t482 = a46, t483 = a80;
      a12 = o_add(o_add(t481, t482), t483);
      a46 = o_sub(o_add(t481, o_shift(t482, 64)), o_shift(t483, 32));
      a80 = o_add(o_sub(t481, o_shift(t482, 32)), o_shift(t483, 64)); }
    { uint64_t t484 = a63, t485 = a97, t486 = a29;
      a63 = o_add(o_add(t484, t485), t486);
      a97 = o_sub(o_add(t484, o_shift(t485, 64)), o_shift(t486, 32));
      a29 = o_add(o_sub(t484, o_shift(t485, 32)), o_shift(t486, 64)); }
    { uint64_t t487 = a12; a12 = o_add(t487, a63); a63 = o_sub(t487, a63); }
    { uint64_t t488 = a46; a46 = o_add(t488, a97); a97 = o_sub(t488, a97); }
    { uint64_t t489 = a80; a80 = o_add(t489, a29); a29 = o_sub(t489, a29); }
    { uint64_t t490 = a24, t491 = a58, t492 = a92;
      a24 = o_add(o_add(t490, t491), t492);
      a58 = o_sub(o_add(t490, o_shift(t491, 64)), o_shift(t492, 32));
      a92 = o_add(o_sub(t490, o_shift(t491, 32)), o_shift(t492, 64)); }
    { uint64_t t493 = a75, t494 = a7, t495 = a41;
      a75 = o_add(o_add(t493, t494), t495);
      a7 = o_sub(o_add(t493, o_shift(t494, 64)), o_shift(t495, 32));
      a41 = o_add(o_sub(t493, o_shift(t494, 32)), o_shift(t495, 64)); }
    { uint64_t t496 = a24; a24 = o_add(t496, a75); a75 = o_sub(t496, a75); }
    { uint64_t t497 = a58; a58 = o_add(t497, a7); a7 = o_sub(t497, a7); }
    { uint64_t t498 = a92; a92 = o_add(t498, a41); a41 = o_sub(t498, a41); }
    { uint64_t t499 = a90, t500 = a22, t501 = a56;
      a90 = o_add(o_add(t499, t500), t501);
      a22 = o_sub(o_add(t499, o_shift(t500, 64)), o_shift(t501, 32));
      a56 = o_add(o_sub(t499, o_shift(t500, 32)), o_shift(t501, 64)); }
    { uint64_t t502 = a39, t503 = a73, t504 = a5;
      a39 = o_add(o_add(t502, t503), t504);
      a73 = o_sub(o_add(t502, o_shift(t503, 64)), o_shift(t504, 32));
      a5 = o_add(o_sub(t502, o_shift(t503, 32)), o_shift(t504, 64)); }
    { uint64_t t505 = a90; a90 = o_add(t505, a39); a39 = o_sub(t505, a39); }
    { uint64_t t506 = a22; a22 = o_add(t506, a73); a73 = o_sub(t506, a73); }
    { uint64_t t507 = a56; a56 = o_add(t507, a5); a5 = o_sub(t507, a5); }
    { uint64_t t508 = a84, t509 = a16, t510 = a50;
      a84 = o_add(o_add(t508, t509), t510);
      a16 = o_sub(o_add(t508, o_shift(t509, 64)), o_shift(t510, 32));
      a50 = o_add(o_sub(t508, o_shift(t509, 32)), o_shift(t510, 64)); }
    { uint64_t t511 = a33, t512 = a67, t513 = a101;
      a33 = o_add(o_add(t511, t512), t513);
      a67 = o_sub(o_add(t511, o_shift(t512, 64)), o_shift(t513, 32));
      a101 = o_add(o_sub(t511, o_shift(t512, 32)), o_shift(t513, 64)); }
    { uint64_t t514 = a84; a84 = o_add(t514, a33); a33 = o_sub(t514, a33); }
    { uint64_t t515 = a16; a16 = o_add(t515, a67); a67 = o_sub(t515, a67); }
    { uint64_t t516 = a50; a50 = o_add(t516, a101); a101 = o_sub(t516, a101); }
    { uint64_t t517 = a54, t518 = a88, t519 = a20;
      a54 = o_add(o_add(t517, t518), t519);
      a88 = o_sub(o_add(t517, o_shift(t518, 64)), o_shift(t519, 32));
      a20 = o_add(o_sub(t517, o_shift(t518, 32)), o_shift(t519, 64)); }
    { uint64_t t520 = a3, t521 = a37, t522 = a71;
      a3 = o_add(o_add(t520, t521), t522);
      a37 = o_sub(o_add(t520, o_shift(t521, 64)), o_shift(t522, 32));
      a71 = o_add(o_sub(t520, o_shift(t521, 32)), o_shift(t522, 64)); }
    { uint64_t t523 = a54; a54 = o_add(t523, a3); a3 = o_sub(t523, a3); }
    { uint64_t t524 = a88; a88 = o_add(t524, a37); a37 = o_sub(t524, a37); }
    { uint64_t t525 = a20; a20 = o_add(t525, a71); a71 = o_sub(t525, a71); }
    { uint64_t t526 = a42, t527 = a76, t528 = a8;
      a42 = o_add(o_add(t526, t527), t528);
      a76 = o_sub(o_add(t526, o_shift(t527, 64)), o_shift(t528, 32));
      a8 = o_add(o_sub(t526, o_shift(t527, 32)), o_shift(t528, 64)); }
    { uint64_t t529 = a93, t530 = a25, t531 = a59;
      a93 = o_add(o_add(t529, t530), t531);
      a25 = o_sub(o_add(t529, o_shift(t530, 64)), o_shift(t531, 32));
      a59 = o_add(o_sub(t529, o_shift(t530, 32)), o_shift(t531, 64)); }
    { uint64_t t532 = a42; a42 = o_add(t532, a93); a93 = o_sub(t532, a93); }
    { uint64_t t533 = a76; a76 = o_add(t533, a25); a25 = o_sub(t533, a25); }
    { uint64_t t534 = a8; a8 = o_add(t534, a59); a59 = o_sub(t534, a59); }
    { uint64_t t535 = a18, t536 = a52, t537 = a86;
      a18 = o_add(o_add(t535, t536), t537);
      a52 = o_sub(o_add(t535, o_shift(t536, 64)), o_shift(t537, 32));
      a86 = o_add(o_sub(t535, o_shift(t536, 32)), o_shift(t537, 64)); }
    { uint64_t t538 = a69, t539 = a1, t540 = a35;
      a69 = o_add(o_add(t538, t539), t540);
      a1 = o_sub(o_add(t538, o_shift(t539, 64)), o_shift(t540, 32));
      a35 = o_add(o_sub(t538, o_shift(t539, 32)), o_shift(t540, 64)); }
    { uint64_t t541 = a18; a18 = o_add(t541, a69); a69 = o_sub(t541, a69); }
    { uint64_t t542 = a52; a52 = o_add(t542, a1); a1 = o_sub(t542, a1); }
    { uint64_t t543 = a86; a86 = o_add(t543, a35); a35 = o_sub(t543, a35); }
    v[0] = a0;
    v[1] = a91;
    v[2] = a32;
    v[3] = a87;
    v[4] = a64;
    v[5] = a65;
    v[6] = a96;
    v[7] = a61;
    v[8] = a26;
    v[9] = a21;
    v[10] = a46;
    v[11] = a41;
    v[12] = a90;
    v[13] = a67;
    v[14] = a20;
    v[15] = a93;
    v[16] = a52;
    v[17] = a17;
    v[18] = a6;
    v[19] = a49;
    v[20] = a2;
    v[21] = a81;
    v[22] = a82;
    v[23] = a11;
    v[24] = a78;
    v[25] = a43;
    v[26] = a38;
    v[27] = a63;
    v[28] = a58;
    v[29] = a5;
    v[30] = a84;
    v[31] = a37;
    v[32] = a8;
    v[33] = a69;
    v[34] = a34;
    v[35] = a23;
    v[36] = a66;
    v[37] = a19;
    v[38] = a98;
    v[39] = a99;
    v[40] = a28;
    v[41] = a95;
    v[42] = a60;
    v[43] = a55;
    v[44] = a80;
    v[45] = a75;
    v[46] = a22;
    v[47] = a101;
    v[48] = a54;
    v[49] = a25;
    v[50] = a86;
    v[51] = a51;
    v[52] = a40;
    v[53] = a83;
    v[54] = a36;
    v[55] = a13;
    v[56] = a14;
    v[57] = a45;
    v[58] = a10;
    v[59] = a77;
    v[60] = a72;
    v[61] = a97;
    v[62] = a92;
    v[63] = a39;
    v[64] = a16;
    v[65] = a71;
    v[66] = a42;
    v[67] = a1;
    v[68] = a68;
    v[69] = a57;
    v[70] = a100;
    v[71] = a53;
    v[72] = a30;
    v[73] = a31;
    v[74] = a62;
    v[75] = a27;
    v[76] = a94;
    v[77] = a89;
    v[78] = a12;
    v[79] = a7;
    v[80] = a56;
    v[81] = a33;
    v[82] = a88;
    v[83] = a59;
    v[84] = a18;
    v[85] = a85;
    v[86] = a74;
    v[87] = a15;
    v[88] = a70;
    v[89] = a47;
    v[90] = a48;
    v[91] = a79;
    v[92] = a44;
    v[93] = a9;
    v[94] = a4;
    v[95] = a29;
    v[96] = a24;
    v[97] = a73;
    v[98] = a50;
    v[99] = a3;
    v[100] = a76;
    v[101] = a35;
}

static void o_ntt_120(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33], a34 = v[34], a35 = v[35], a36 = v[36], a37 = v[37], a38 = v[38], a39 = v[39], a40 = v[40], a41 = v[41], a42 = v[42], a43 = v[43], a44 = v[44], a45 = v[45], a46 = v[46], a47 = v[47], a48 = v[48], a49 = v[49], a50 = v[50], a51 = v[51], a52 = v[52], a53 = v[53], a54 = v[54], a55 = v[55], a56 = v[56], a57 = v[57], a58 = v[58], a59 = v[59], a60 = v[60], a61 = v[61], a62 = v[62], a63 = v[63], a64 = v[64], a65 = v[65], a66 = v[66], a67 = v[67], a68 = v[68], a69 = v[69], a70 = v[70], a71 = v[71], a72 = v[72], a73 = v[73], a74 = v[74], a75 = v[75], a76 = v[76], a77 = v[77], a78 = v[78], a79 = v[79], a80 = v[80], a81 = v[81], a82 = v[82], a83 = v[83], a84 = v[84], a85 = v[85], a86 = v[86], a87 = v[87], a88 = v[88], a89 = v[89], a90 = v[90], a91 = v[91], a92 = v[92], a93 = v[93], a94 = v[94], a95 = v[95], a96 = v[96], a97 = v[97], a98 = v[98], a99 = v[99], a100 = v[100], a101 = v[101], a102 = v[102], a103 = v[103], a104 = v[104], a105 = v[105], a106 = v[106], a107 = v[107], a108 = v[108], a109 = v[109], a110 = v[110], a111 = v[111], a112 = v[112], a113 = v[113], a114 = v[114], a115 = v[115], a116 = v[116], a117 = v[117], a118 = v[118], a119 = v[119];
    { uint64_t t1 = a24; a24 = o_add(t1, a96); a96 = o_sub(t1, a96); }
    { uint64_t t2 = a72; a72 = o_add(t2, a48); a48 = o_sub(t2, a48); }
    a48 = o_shift(a48, 48);
    { uint64_t t3 = a24; a24 = o_add(t3, a72); a72 = o_sub(t3, a72); }
    { uint64_t t4 = a96; a96 = o_add(t4, a48); a48 = o_sub(t4, a48); }
    uint64_t t5 = a0;
    a0 = o_add(a0, a24);
    a24 = o_mul(a24, 4611686017353646080ULL);
    a96 = o_mul(a96, 16181989089180173841ULL);
    a72 = o_mul(a72, 5818851782451133869ULL);
    a48 = o_mul(a48, 11322249509082494407ULL);
    a24 = o_add(a24, t5);
    { uint64_t t6 = a24; a24 = o_add(t6, a72); a72 = o_sub(t6, a72); }
    { uint64_t t7 = a48; a48 = o_add(t7, a96); a96 = o_sub(t7, a96); }
    a96 = o_shift(a96, 48);
    { uint64_t t8 = a24; a24 = o_add(t8, a48); a48 = o_sub(t8, a48); }
    { uint64_t t9 = a72; a72 = o_add(t9, a96); a96 = o_sub(t9, a96); }
    { uint64_t t10 = a84; a84 = o_add(t10, a36); a36 = o_sub(t10, a36); }
    { uint64_t t11 = a12; a12 = o_add(t11, a108); a108 = o_sub(t11, a108); }
    a108 = o_shift(a108, 48);
    { uint64_t t12 = a84; a84 = o_add(t12, a12); a12 = o_sub(t12, a12); }
    { uint64_t t13 = a36; a36 = o_add(t13, a108); a108 = o_sub(t13, a108); }
    uint64_t t14 = a60;
    a60 = o_add(a60, a84);
    a84 = o_mul(a84, 4611686017353646080ULL);
    a36 = o_mul(a36, 16181989089180173841ULL);
    a12 = o_mul(a12, 5818851782451133869ULL);
    a108 = o_mul(a108, 11322249509082494407ULL);
    a84 = o_add(a84, t14);
    { uint64_t t15 = a84; a84 = o_add(t15, a12); a12 = o_sub(t15, a12); }
    { uint64_t t16 = a108; a108 = o_add(t16, a36); a36 = o_sub(t16, a36); }
    a36 = o_shift(a36, 48);
    { uint64_t t17 = a84; a84 = o_add(t17, a108); a108 = o_sub(t17, a108); }
    { uint64_t t18 = a12; a12 = o_add(t18, a36); a36 = o_sub(t18, a36); }
    { uint64_t t19 = a0; a0 = o_add(t19, a60); a60 = o_sub(t19, a60); }
    { uint64_t t20 = a24; a24 = o_add(t20, a84); a84 = o_sub(t20, a84); }
    { uint64_t t21 = a72; a72 = o_add(t21, a12); a12 = o_sub(t21, a12); }
    { uint64_t t22 = a96; a96 = o_add(t22, a36); a36 = o_sub(t22, a36); }
    { uint64_t t23 = a48; a48 = o_add(t23, a108); a108 = o_sub(t23, a108); }
    { uint64_t t24 = a25; a25 = o_add(t24, a97); a97 = o_sub(t24, a97); }
    { uint64_t t25 = a73; a73 = o_add(t25, a49); a49 = o_sub(t25, a49); }
    a49 = o_shift(a49, 48);
    { uint64_t t26 = a25; a25 = o_add(t26, a73); a73 = o_sub(t26, a73); }
    { uint64_t t27 = a97; a97 = o_add(t27, a49); a49 = o_sub(t27, a49); }
    uint64_t t28 = a1;
    a1 = o_add(a1, a25);
    a25 = o_mul(a25, 4611686017353646080ULL);
    a97 = o_mul(a97, 16181989089180173841ULL);
    a73 = o_mul(a73, 5818851782451133869ULL);
    a49 = o_mul(a49, 11322249509082494407ULL);
    a25 = o_add(a25, t28);
    { uint64_t t29 = a25; a25 = o_add(t29, a73); a73 = o_sub(t29, a73); }
    { uint64_t t30 = a49; a49 = o_add(t30, a97); a97 = o_sub(t30, a97); }
    a97 = o_shift(a97, 48);
    { uint64_t t31 = a25; a25 = o_add(t31, a49); a49 = o_sub(t31, a49); }
    { uint64_t t32 = a73; a73 = o_add(t32, a97); a97 = o_sub(t32, a97); }
    { uint64_t t33 = a85; a85 = o_add(t33, a37); a37 = o_sub(t33, a37); }
    { uint64_t t34 = a13; a13 = o_add(t34, a109); a109 = o_sub(t34, a109); }
    a109 = o_shift(a109, 48);
    { uint64_t t35 = a85; a85 = o_add(t35, a13); a13 = o_sub(t35, a13); }
    { uint64_t t36 = a37; a37 = o_add(t36, a109); a109 = o_sub(t36, a109); }
    uint64_t t37 = a61;
    a61 = o_add(a61, a85);
    a85 = o_mul(a85, 4611686017353646080ULL);
    a37 = o_mul(a37, 16181989089180173841ULL);
    a13 = o_mul(a13, 5818851782451133869ULL);
    a109 = o_mul(a109, 11322249509082494407ULL);
    a85 = o_add(a85, t37);
    { uint64_t t38 = a85; a85 = o_add(t38, a13); a13 = o_sub(t38, a13); }
    { uint64_t t39 = a109; a109 = o_add(t39, a37); a37 = o_sub(t39, a37); }
    a37 = o_shift(a37, 48);
    { uint64_t t40 = a85; a85 = o_add(t40, a109); a109 = o_sub(t40, a109); }
    { uint64_t t41 = a13; a13 = o_add(t41, a37); a37 = o_sub(t41, a37); }
    { uint64_t t42 = a1; a1 = o_add(t42, a61); a61 = o_sub(t42, a61); }
    { uint64_t t43 = a25; a25 = o_add(t43, a85); a85 = o_sub(t43, a85); }
    { uint64_t t44 = a73; a73 = o_add(t44, a13); a13 = o_sub(t44, a13); }
    { uint64_t t45 = a97; a97 = o_add(t45, a37); a37 = o_sub(t45, a37); }
    { uint64_t t46 = a49; a49 = o_add(t46, a109); a109 = o_sub(t46, a109); }
    { uint64_t t47 = a26; a26 = o_add(t47, a98); a98 = o_sub(t47, a98); }
    { uint64_t t48 = a74; a74 = o_add(t48, a50); a50 = o_sub(t48, a50); }
    a50 = o_shift(a50, 48);
    { uint64_t t49 = a26; a26 = o_add(t49, a74); a74 = o_sub(t49, a74); }
    { uint64_t t50 = a98; a98 = o_add(t50, a50); a50 = o_sub(t50, a50); }
    uint64_t t51 = a2;
    a2 = o_add(a2, a26);
    a26 = o_mul(a26, 4611686017353646080ULL);
    a98 = o_mul(a98, 16181989089180173841ULL);
    a74 = o_mul(a74, 5818851782451133869ULL);
    a50 = o_mul(a50, 11322249509082494407ULL);
    a26 = o_add(a26, t51);
    { uint64_t t52 = a26; a26 = o_add(t52, a74); a74 = o_sub(t52, a74); }
    { uint64_t t53 = a50; a50 = o_add(t53, a98); a98 = o_sub(t53, a98); }
    a98 = o_shift(a98, 48);
    { uint64_t t54 = a26; a26 = o_add(t54, a50); a50 = o_sub(t54, a50); }
    { uint64_t t55 = a74; a74 = o_add(t55, a98); a98 = o_sub(t55, a98); }
    { uint64_t t56 = a86; a86 = o_add(t56, a38); a38 = o_sub(t56, a38); }
    { uint64_t t57 = a14; a14 = o_add(t57, a110); a110 = o_sub(t57, a110); }
    a110 = o_shift(a110, 48);
    { uint64_t t58 = a86; a86 = o_add(t58, a14); a14 = o_sub(t58, a14); }
    { uint64_t t59 = a38; a38 = o_add(t59, a110); a110 = o_sub(t59, a110); }
    uint64_t t60 = a62;
    a62 = o_add(a62, a86);
    a86 = o_mul(a86, 4611686017353646080ULL);
    a38 = o_mul(a38, 16181989089180173841ULL);
    a14 = o_mul(a14, 5818851782451133869ULL);
    a110 = o_mul(a110, 11322249509082494407ULL);
    a86 = o_add(a86, t60);
    { uint64_t t61 = a86; a86 = o_add(t61, a14); a14 = o_sub(t61, a14); }
    { uint64_t t62 = a110; a110 = o_add(t62, a38); a38 = o_sub(t62, a38); }
    a38 = o_shift(a38, 48);
    { uint64_t t63 = a86; a86 = o_add(t63, a110); a110 = o_sub(t63, a110); }
    { uint64_t t64 = a14; a14 = o_add(t64, a38); a38 = o_sub(t64, a38); }
    { uint64_t t65 = a2; a2 = o_add(t65, a62); a62 = o_sub(t65, a62); }
    { uint64_t t66 = a26; a26 = o_add(t66, a86); a86 = o_sub(t66, a86); }
    { uint64_t t67 = a74; a74 = o_add(t67, a14); a14 = o_sub(t67, a14); }
    { uint64_t t68 = a98; a98 = o_add(t68, a38); a38 = o_sub(t68, a38); }
    { uint64_t t69 = a50; a50 = o_add(t69, a110); a110 = o_sub(t69, a110); }
    { uint64_t t70 = a27; a27 = o_add(t70, a99); a99 = o_sub(t70, a99); }
    { uint64_t t71 = a75; a75 = o_add(t71, a51); a51 = o_sub(t71, a51); }
    a51 = o_shift(a51, 48);
    { uint64_t t72 = a27; a27 = o_add(t72, a75); a75 = o_sub(t72, a75); }
    { uint64_t t73 = a99; a99 = o_add(t73, a51); a51 = o_sub(t73, a51); }
    uint64_t t74 = a3;
    a3 = o_add(a3, a27);
    a27 = o_mul(a27, 4611686017353646080ULL);
    a99 = o_mul(a99, 16181989089180173841ULL);
    a75 = o_mul(a75, 5818851782451133869ULL);
    a51 = o_mul(a51, 11322249509082494407ULL);
    a27 = o_add(a27, t74);
    { uint64_t t75 = a27; a27 = o_add(t75, a75); a75 = o_sub(t75, a75); }
    { uint64_t t76 = a51; a51 = o_add(t76, a99); a99 = o_sub(t76, a99); }
    a99 = o_shift(a99, 48);
    { uint64_t t77 = a27; a27 = o_add(t77, a51); a51 = o_sub(t77, a51); }
    { uint64_t t78 = a75; a75 = o_add(t78, a99); a99 = o_sub(t78, a99); }
    { uint64_t t79 = a87; a87 = o_add(t79, a39); a39 = o_sub(t79, a39); }
    { uint64_t t80 = a15; a15 = o_add(t80, a111); a111 = o_sub(t80, a111); }
    a111 = o_shift(a111, 48);
    { uint64_t t81 = a87; a87 = o_add(t81, a15); a15 = o_sub(t81, a15); }
    { uint64_t t82 = a39; a39 = o_add(t82, a111); a111 = o_sub(t82, a111); }
    uint64_t t83 = a63;
    a63 = o_add(a63, a87);
    a87 = o_mul(a87, 4611686017353646080ULL);
    a39 = o_mul(a39, 16181989089180173841ULL);
    a15 = o_mul(a15, 5818851782451133869ULL);
    a111 = o_mul(a111, 11322249509082494407ULL);
    a87 = o_add(a87, t83);
    { uint64_t t84 = a87; a87 = o_add(t84, a15); a15 = o_sub(t84, a15); }
    { uint64_t t85 = a111; a111 = o_add(t85, a39); a39 = o_sub(t85, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t86 = a87; a87 = o_add(t86, a111); a111 = o_sub(t86, a111); }
    { uint64_t t87 = a15; a15 = o_add(t87, a39); a39 = o_sub(t87, a39); }
    { uint64_t t88 = a3; a3 = o_add(t88, a63); a63 = o_sub(t88, a63); }
    { uint64_t t89 = a27; a27 = o_add(t89, a87); a87 = o_sub(t89, a87); }
    { uint64_t t90 = a75; a75 = o_add(t90, a15); a15 = o_sub(t90, a15); }
    { uint64_t t91 = a99; a99 = o_add(t91, a39); a39 = o_sub(t91, a39); }
    { uint64_t t92 = a51; a51 = o_add(t92, a111); a111 = o_sub(t92, a111); }
    { uint64_t t93 = a28; a28 = o_add(t93, a100); a100 = o_sub(t93, a100); }
    { uint64_t t94 = a76; a76 = o_add(t94, a52); a52 = o_sub(t94, a52); }
    a52 = o_shift(a52, 48);
    { uint64_t t95 = a28; a28 = o_add(t95, a76); a76 = o_sub(t95, a76); }
    { uint64_t t96 = a100; a100 = o_add(t96, a52); a52 = o_sub(t96, a52); }
    uint64_t t97 = a4;
    a4 = o_add(a4, a28);
    a28 = o_mul(a28, 4611686017353646080ULL);
    a100 = o_mul(a100, 16181989089180173841ULL);
    a76 = o_mul(a76, 5818851782451133869ULL);
    a52 = o_mul(a52, 11322249509082494407ULL);
    a28 = o_add(a28, t97);
    { uint64_t t98 = a28; a28 = o_add(t98, a76); a76 = o_sub(t98, a76); }
    { uint64_t t99 = a52; a52 = o_add(t99, a100); a100 = o_sub(t99, a100); }
    a100 = o_shift(a100, 48);
    { uint64_t t100 = a28; a28 = o_add(t100, a52); a52 = o_sub(t100, a52); }
    { uint64_t t101 = a76; a76 = o_add(t101, a100); a100 = o_sub(t101, a100); }
    { uint64_t t102 = a88; a88 = o_add(t102, a40); a40 = o_sub(t102, a40); }
    { uint64_t t103 = a16; a16 = o_add(t103, a112); a112 = o_sub(t103, a112); }
    a112 = o_shift(a112, 48);
    { uint64_t t104 = a88; a88 = o_add(t104, a16); a16 = o_sub(t104, a16); }
    { uint64_t t105 = a40; a40 = o_add(t105, a112); a112 = o_sub(t105, a112); }
    uint64_t t106 = a64;
    a64 = o_add(a64, a88);
    a88 = o_mul(a88, 4611686017353646080ULL);
    a40 = o_mul(a40, 16181989089180173841ULL);
    a16 = o_mul(a16, 5818851782451133869ULL);
    a112 = o_mul(a112, 11322249509082494407ULL);
    a88 = o_add(a88, t106);
    { uint64_t t107 = a88; a88 = o_add(t107, a16); a16 = o_sub(t107, a16); }
    { uint64_t t108 = a112; a112 = o_add(t108, a40); a40 = o_sub(t108, a40); }
    a40 = o_shift(a40, 48);
    { uint64_t t109 = a88; a88 = o_add(t109, a112); a112 = o_sub(t109, a112); }
    { uint64_t t110 = a16; a16 = o_add(t110, a40); a40 = o_sub(t110, a40); }
    { uint64_t t111 = a4; a4 = o_add(t111, a64); a64 = o_sub(t111, a64); }
    { uint64_t t112 = a28; a28 = o_add(t112, a88); a88 = o_sub(t112, a88); }
    { uint64_t t113 = a76; a76 = o_add(t113, a16); a16 = o_sub(t113, a16); }
    { uint64_t t114 = a100; a100 = o_add(t114, a40); a40 = o_sub(t114, a40); }
    { uint64_t t115 = a52; a52 = o_add(t115, a112); a112 = o_sub(t115, a112); }
    { uint64_t t116 = a29; a29 = o_add(t116, a101); a101 = o_sub(t116, a101); }
    { uint64_t t117 = a77; a77 = o_add(t117, a53); a53 = o_sub(t117, a53); }
    a53 = o_shift(a53, 48);
    { uint64_t t118 = a29; a29 = o_add(t118, a77); a77 = o_sub(t118, a77); }
    { uint64_t t119 = a101; a101 = o_add(t119, a53); a53 = o_sub(t119, a53); }
    uint64_t t120 = a5;
    a5 = o_add(a5, a29);
    a29 = o_mul(a29, 4611686017353646080ULL);
    a101 = o_mul(a101, 16181989089180173841ULL);
    a77 = o_mul(a77, 5818851782451133869ULL);
    a53 = o_mul(a53, 11322249509082494407ULL);
    a29 = o_add(a29, t120);
    { uint64_t t121 = a29; a29 = o_add(t121, a77); a77 = o_sub(t121, a77); }
    { uint64_t t122 = a53; a53 = o_add(t122, a101); a101 = o_sub(t122, a101); }
    a101 = o_shift(a101, 48);
    { uint64_t t123 = a29; a29 = o_add(t123, a53); a53 = o_sub(t123, a53); }
    { uint64_t t124 = a77; a77 = o_add(t124, a101); a101 = o_sub(t124, a101); }
    { uint64_t t125 = a89; a89 = o_add(t125, a41); a41 = o_sub(t125, a41); }
    { uint64_t t126 = a17; a17 = o_add(t126, a113); a113 = o_sub(t126, a113); }
    a113 = o_shift(a113, 48);
    { uint64_t t127 = a89; a89 = o_add(t127, a17); a17 = o_sub(t127, a17); }
    { uint64_t t128 = a41; a41 = o_add(t128, a113); a113 = o_sub(t128, a113); }
    uint64_t t129 = a65;
    a65 = o_add(a65, a89);
    a89 = o_mul(a89, 4611686017353646080ULL);
    a41 = o_mul(a41, 16181989089180173841ULL);
    a17 = o_mul(a17, 5818851782451133869ULL);
    a113 = o_mul(a113, 11322249509082494407ULL);
    a89 = o_add(a89, t129);
    { uint64_t t130 = a89; a89 = o_add(t130, a17); a17 = o_sub(t130, a17); }
    { uint64_t t131 = a113; a113 = o_add(t131, a41); a41 = o_sub(t131, a41); }
    a41 = o_shift(a41, 48);
    { uint64_t t132 = a89; a89 = o_add(t132, a113); a113 = o_sub(t132, a113); }
    { uint64_t t133 = a17; a17 = o_add(t133, a41); a41 = o_sub(t133, a41); }
    { uint64_t t134 = a5; a5 = o_add(t134, a65); a65 = o_sub(t134, a65); }
    { uint64_t t135 = a29; a29 = o_add(t135, a89); a89 = o_sub(t135, a89); }
    { uint64_t t136 = a77; a77 = o_add(t136, a17); a17 = o_sub(t136, a17); }
    { uint64_t t137 = a101; a101 = o_add(t137, a41); a41 = o_sub(t137, a41); }
    { uint64_t t138 = a53; a53 = o_add(t138, a113); a113 = o_sub(t138, a113); }
    { uint64_t t139 = a30; a30 = o_add(t139, a102); a102 = o_sub(t139, a102); }
    { uint64_t t140 = a78; a78 = o_add(t140, a54); a54 = o_sub(t140, a54); }
    a54 = o_shift(a54, 48);
    { uint64_t t141 = a30; a30 = o_add(t141, a78); a78 = o_sub(t141, a78); }
    { uint64_t t142 = a102; a102 = o_add(t142, a54); a54 = o_sub(t142, a54); }
    uint64_t t143 = a6;
    a6 = o_add(a6, a30);
    a30 = o_mul(a30, 4611686017353646080ULL);
    a102 = o_mul(a102, 16181989089180173841ULL);
    a78 = o_mul(a78, 5818851782451133869ULL);
    a54 = o_mul(a54, 11322249509082494407ULL);
    a30 = o_add(a30, t143);
    { uint64_t t144 = a30; a30 = o_add(t144, a78); a78 = o_sub(t144, a78); }
    { uint64_t t145 = a54; a54 = o_add(t145, a102); a102 = o_sub(t145, a102); }
    a102 = o_shift(a102, 48);
    { uint64_t t146 = a30; a30 = o_add(t146, a54); a54 = o_sub(t146, a54); }
    { uint64_t t147 = a78; a78 = o_add(t147, a102); a102 = o_sub(t147, a102); }
    { uint64_t t148 = a90; a90 = o_add(t148, a42); a42 = o_sub(t148, a42); }
    { uint64_t t149 = a18; a18 = o_add(t149, a114); a114 = o_sub(t149, a114); }
    a114 = o_shift(a114, 48);
    { uint64_t t150 = a90; a90 = o_add(t150, a18); a18 = o_sub(t150, a18); }
    { uint64_t t151 = a42; a42 = o_add(t151, a114); a114 = o_sub(t151, a114); }
    uint64_t t152 = a66;
    a66 = o_add(a66, a90);
    a90 = o_mul(a90, 4611686017353646080ULL);
    a42 = o_mul(a42, 16181989089180173841ULL);
    a18 = o_mul(a18, 5818851782451133869ULL);
    a114 = o_mul(a114, 11322249509082494407ULL);
    a90 = o_add(a90, t152);
    { uint64_t t153 = a90; a90 = o_add(t153, a18); a18 = o_sub(t153, a18); }
    { uint64_t t154 = a114; a114 = o_add(t154, a42); a42 = o_sub(t154, a42); }
    a42 = o_shift(a42, 48);
    { uint64_t t155 = a90; a90 = o_add(t155, a114); a114 = o_sub(t155, a114); }
    { uint64_t t156 = a18; a18 = o_add(t156, a42); a42 = o_sub(t156, a42); }
    { uint64_t t157 = a6; a6 = o_add(t157, a66); a66 = o_sub(t157, a66); }
    { uint64_t t158 = a30; a30 = o_add(t158, a90); a90 = o_sub(t158, a90); }
    { uint64_t t159 = a78; a78 = o_add(t159, a18); a18 = o_sub(t159, a18); }
    { uint64_t t160 = a102; a102 = o_add(t160, a42); a42 = o_sub(t160, a42); }
    { uint64_t t161 = a54; a54 = o_add(t161, a114); a114 = o_sub(t161, a114); }
    { uint64_t t162 = a31; a31 = o_add(t162, a103); a103 = o_sub(t162, a103); }
    { uint64_t t163 = a79; a79 = o_add(t163, a55); a55 = o_sub(t163, a55); }
    a55 = o_shift(a55, 48);
    { uint64_t t164 = a31; a31 = o_add(t164, a79); a79 = o_sub(t164, a79); }
    { uint64_t t165 = a103; a103 = o_add(t165, a55); a55 = o_sub(t165, a55); }
    uint64_t t166 = a7;
    a7 = o_add(a7, a31);
    a31 = o_mul(a31, 4611686017353646080ULL);
    a103 = o_mul(a103, 16181989089180173841ULL);
    a79 = o_mul(a79, 5818851782451133869ULL);
    a55 = o_mul(a55, 11322249509082494407ULL);
    a31 = o_add(a31, t166);
    { uint64_t t167 = a31; a31 = o_add(t167, a79); a79 = o_sub(t167, a79); }
    { uint64_t t168 = a55; a55 = o_add(t168, a103); a103 = o_sub(t168, a103); }
    a103 = o_shift(a103, 48);
    { uint64_t t169 = a31; a31 = o_add(t169, a55); a55 = o_sub(t169, a55); }
    { uint64_t t170 = a79; a79 = o_add(t170, a103); a103 = o_sub(t170, a103); }
    { uint64_t t171 = a91; a91 = o_add(t171, a43); a43 = o_sub(t171, a43); }
    { uint64_t t172 = a19; a19 = o_add(t172, a115); a115 = o_sub(t172, a115); }
    a115 = o_shift(a115, 48);
    { uint64_t t173 = a91; a91 = o_add(t173, a19); a19 = o_sub(t173, a19); }
    { uint64_t t174 = a43; a43 = o_add(t174, a115); a115 = o_sub(t174, a115); }
    uint64_t t175 = a67;
    a67 = o_add(a67, a91);
    a91 = o_mul(a91, 4611686017353646080ULL);
    a43 = o_mul(a43, 16181989089180173841ULL);
    a19 = o_mul(a19, 5818851782451133869ULL);
    a115 = o_mul(a115, 11322249509082494407ULL);
    a91 = o_add(a91, t175);
    { uint64_t t176 = a91; a91 = o_add(t176, a19); a19 = o_sub(t176, a19); }
    { uint64_t t177 = a115; a115 = o_add(t177, a43); a43 = o_sub(t177, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t178 = a91; a91 = o_add(t178, a115); a115 = o_sub(t178, a115); }
    { uint64_t t179 = a19; a19 = o_add(t179, a43); a43 = o_sub(t179, a43); }
    { uint64_t t180 = a7; a7 = o_add(t180, a67); a67 = o_sub(t180, a67); }
    { uint64_t t181 = a31; a31 = o_add(t181, a91); a91 = o_sub(t181, a91); }
    { uint64_t t182 = a79; a79 = o_add(t182, a19); a19 = o_sub(t182, a19); }
    { uint64_t t183 = a103; a103 = o_add(t183, a43); a43 = o_sub(t183, a43); }
    { uint64_t t184 = a55; a55 = o_add(t184, a115); a115 = o_sub(t184, a115); }
    { uint64_t t185 = a32; a32 = o_add(t185, a104); a104 = o_sub(t185, a104); }
    { uint64_t t186 = a80; a80 = o_add(t186, a56); a56 = o_sub(t186, a56); }
    a56 = o_shift(a56, 48);
    { uint64_t t187 = a32; a32 = o_add(t187, a80); a80 = o_sub(t187, a80); }
    { uint64_t t188 = a104; a104 = o_add(t188, a56); a56 = o_sub(t188, a56); }
    uint64_t t189 = a8;
    a8 = o_add(a8, a32);
    a32 = o_mul(a32, 4611686017353646080ULL);
    a104 = o_mul(a104, 16181989089180173841ULL);
    a80 = o_mul(a80, 5818851782451133869ULL);
    a56 = o_mul(a56, 11322249509082494407ULL);
    a32 = o_add(a32, t189);
    { uint64_t t190 = a32; a32 = o_add(t190, a80); a80 = o_sub(t190, a80); }
    { uint64_t t191 = a56; a56 = o_add(t191, a104); a104 = o_sub(t191, a104); }
    a104 = o_shift(a104, 48);
    { uint64_t t192 = a32; a32 = o_add(t192, a56); a56 = o_sub(t192, a56); }
    { uint64_t t193 = a80; a80 = o_add(t193, a104); a104 = o_sub(t193, a104); }
    { uint64_t t194 = a92; a92 = o_add(t194, a44); a44 = o_sub(t194, a44); }
    { uint64_t t195 = a20; a20 = o_add(t195, a116); a116 = o_sub(t195, a116); }
    a116 = o_shift(a116, 48);
    { uint64_t t196 = a92; a92 = o_add(t196, a20); a20 = o_sub(t196, a20); }
    { uint64_t t197 = a44; a44 = o_add(t197, a116); a116 = o_sub(t197, a116); }
    uint64_t t198 = a68;
    a68 = o_add(a68, a92);
    a92 = o_mul(a92, 4611686017353646080ULL);
    a44 = o_mul(a44, 16181989089180173841ULL);
    a20 = o_mul(a20, 5818851782451133869ULL);
    a116 = o_mul(a116, 11322249509082494407ULL);
    a92 = o_add(a92, t198);
    { uint64_t t199 = a92; a92 = o_add(t199, a20); a20 = o_sub(t199, a20); }
    { uint64_t t200 = a116; a116 = o_add(t200, a44); a44 = o_sub(t200, a44); }
    a44 = o_shift(a44, 48);
    { uint64_t t201 = a92; a92 = o_add(t201, a116); a116 = o_sub(t201, a116); }
    { uint64_t t202 = a20; a20 = o_add(t202, a44); a44 = o_sub(t202, a44); }
    { uint64_t t203 = a8; a8 = o_add(t203, a68); a68 = o_sub(t203, a68); }
    { uint64_t t204 = a32; a32 = o_add(t204, a92); a92 = o_sub(t204, a92); }
    { uint64_t t205 = a80; a80 = o_add(t205, a20); a20 = o_sub(t205, a20); }
    { uint64_t t206 = a104; a104 = o_add(t206, a44); a44 = o_sub(t206, a44); }
    { uint64_t t207 = a56; a56 = o_add(t207, a116); a116 = o_sub(t207, a116); }
    { uint64_t t208 = a33; a33 = o_add(t208, a105); a105 = o_sub(t208, a105); }
    { uint64_t t209 = a81; a81 = o_add(t209, a57); a57 = o_sub(t209, a57); }
    a57 = o_shift(a57, 48);
    { uint64_t t210 = a33; a33 = o_add(t210, a81); a81 = o_sub(t210, a81); }
    { uint64_t t211 = a105; a105 = o_add(t211, a57); a57 = o_sub(t211, a57); }
    uint64_t t212 = a9;
    a9 = o_add(a9, a33);
    a33 = o_mul(a33, 4611686017353646080ULL);
    a105 = o_mul(a105, 16181989089180173841ULL);
    a81 = o_mul(a81, 5818851782451133869ULL);
    a57 = o_mul(a57, 11322249509082494407ULL);
    a33 = o_add(a33, t212);
    { uint64_t t213 = a33; a33 = o_add(t213, a81); a81 = o_sub(t213, a81); }
    { uint64_t t214 = a57; a57 = o_add(t214, a105); a105 = o_sub(t214, a105); }
    a105 = o_shift(a105, 48);
    { uint64_t t215 = a33; a33 = o_add(t215, a57); a57 = o_sub(t215, a57); }
    { uint64_t t216 = a81; a81 = o_add(t216, a105); a105 = o_sub(t216, a105); }
    { uint64_t t217 = a93; a93 = o_add(t217, a45); a45 = o_sub(t217, a45); }
    { uint64_t t218 = a21; a21 = o_add(t218, a117); a117 = o_sub(t218, a117); }
    a117 = o_shift(a117, 48);
    { uint64_t t219 = a93; a93 = o_add(t219, a21); a21 = o_sub(t219, a21); }
    { uint64_t t220 = a45; a45 = o_add(t220, a117); a117 = o_sub(t220, a117); }
    uint64_t t221 = a69;
    a69 = o_add(a69, a93);
    a93 = o_mul(a93, 4611686017353646080ULL);
    a45 = o_mul(a45, 16181989089180173841ULL);
    a21 = o_mul(a21, 5818851782451133869ULL);
    a117 = o_mul(a117, 11322249509082494407ULL);
    a93 = o_add(a93, t221);
    { uint64_t t222 = a93; a93 = o_add(t222, a21); a21 = o_sub(t222, a21); }
    { uint64_t t223 = a117; a117 = o_add(t223, a45); a45 = o_sub(t223, a45); }
    a45 = o_shift(a45, 48);
    { uint64_t t224 = a93; a93 = o_add(t224, a117); a117 = o_sub(t224, a117); }
    { uint64_t t225 = a21; a21 = o_add(t225, a45); a45 = o_sub(t225, a45); }
    { uint64_t t226 = a9; a9 = o_add(t226, a69); a69 = o_sub(t226, a69); }
    { uint64_t t227 = a33; a33 = o_add(t227, a93); a93 = o_sub(t227, a93); }
    { uint64_t t228 = a81; a81 = o_add(t228, a21); a21 = o_sub(t228, a21); }
    { uint64_t t229 = a105; a105 = o_add(t229, a45); a45 = o_sub(t229, a45); }
    { uint64_t t230 = a57; a57 = o_add(t230, a117); a117 = o_sub(t230, a117); }
    { uint64_t t231 = a34; a34 = o_add(t231, a106); a106 = o_sub(t231, a106); }
    { uint64_t t232 = a82; a82 = o_add(t232, a58); a58 = o_sub(t232, a58); }
    a58 = o_shift(a58, 48);
    { uint64_t t233 = a34; a34 = o_add(t233, a82); a82 = o_sub(t233, a82); }
    { uint64_t t234 = a106; a106 = o_add(t234, a58); a58 = o_sub(t234, a58); }
    uint64_t t235 = a10;
    a10 = o_add(a10, a34);
    a34 = o_mul(a34, 4611686017353646080ULL);
    a106 = o_mul(a106, 16181989089180173841ULL);
    a82 = o_mul(a82, 5818851782451133869ULL);
    a58 = o_mul(a58, 11322249509082494407ULL);
    a34 = o_add(a34, t235);
    { uint64_t t236 = a34; a34 = o_add(t236, a82); a82 = o_sub(t236, a82); }
    { uint64_t t237 = a58; a58 = o_add(t237, a106); a106 = o_sub(t237, a106); }
    a106 = o_shift(a106, 48);
    { uint64_t t238 = a34; a34 = o_add(t238, a58); a58 = o_sub(t238, a58); }
    { uint64_t t239 = a82; a82 = o_add(t239, a106); a106 = o_sub(t239, a106); }
    { uint64_t t240 = a94; a94 = o_add(t240, a46); a46 = o_sub(t240, a46); }
    { uint64_t t241 = a22; a22 = o_add(t241, a118); a118 = o_sub(t241, a118); }
    a118 = o_shift(a118, 48);
    { uint64_t t242 = a94; a94 = o_add(t242, a22); a22 = o_sub(t242, a22); }
    { uint64_t t243 = a46; a46 = o_add(t243, a118); a118 = o_sub(t243, a118); }
    uint64_t t244 = a70;
    a70 = o_add(a70, a94);
    a94 = o_mul(a94, 4611686017353646080ULL);
    a46 = o_mul(a46, 16181989089180173841ULL);
    a22 = o_mul(a22, 5818851782451133869ULL);
    a118 = o_mul(a118, 11322249509082494407ULL);
    a94 = o_add(a94, t244);
    { uint64_t t245 = a94; a94 = o_add(t245, a22); a22 = o_sub(t245, a22); }
    { uint64_t t246 = a118; a118 = o_add(t246, a46); a46 = o_sub(t246, a46); }
    a46 = o_shift(a46, 48);
    { uint64_t t247 = a94; a94 = o_add(t247, a118); a118 = o_sub(t247, a118); }
    { uint64_t t248 = a22; a22 = o_add(t248, a46); a46 = o_sub(t248, a46); }
    { uint64_t t249 = a10; a10 = o_add(t249, a70); a70 = o_sub(t249, a70); }
    { uint64_t t250 = a34; a34 = o_add(t250, a94); a94 = o_sub(t250, a94); }
    { uint64_t t251 = a82; a82 = o_add(t251, a22); a22 = o_sub(t251, a22); }
    { uint64_t t252 = a106; a106 = o_add(t252, a46); a46 = o_sub(t252, a46); }
    { uint64_t t253 = a58; a58 = o_add(t253, a118); a118 = o_sub(t253, a118); }
    { uint64_t t254 = a35; a35 = o_add(t254, a107); a107 = o_sub(t254, a107); }
    { uint64_t t255 = a83; a83 = o_add(t255, a59); a59 = o_sub(t255, a59); }
    a59 = o_shift(a59, 48);
    { uint64_t t256 = a35; a35 = o_add(t256, a83); a83 = o_sub(t256, a83); }
    { uint64_t t257 = a107; a107 = o_add(t257, a59); a59 = o_sub(t257, a59); }
    uint64_t t258 = a11;
    a11 = o_add(a11, a35);
    a35 = o_mul(a35, 4611686017353646080ULL);
    a107 = o_mul(a107, 16181989089180173841ULL);
    a83 = o_mul(a83, 5818851782451133869ULL);
    a59 = o_mul(a59, 11322249509082494407ULL);
    a35 = o_add(a35, t258);
    { uint64_t t259 = a35; a35 = o_add(t259, a83); a83 = o_sub(t259, a83); }
    { uint64_t t260 = a59; a59 = o_add(t260, a107); a107 = o_sub(t260, a107); }
    a107 = o_shift(a107, 48);
    { uint64_t t261 = a35; a35 = o_add(t261, a59); a59 = o_sub(t261, a59); }
    { uint64_t t262 = a83; a83 = o_add(t262, a107); a107 = o_sub(t262, a107); }
    { uint64_t t263 = a95; a95 = o_add(t263, a47); a47 = o_sub(t263, a47); }
    { uint64_t t264 = a23; a23 = o_add(t264, a119); a119 = o_sub(t264, a119); }
    a119 = o_shift(a119, 48);
    { uint64_t t265 = a95; a95 = o_add(t265, a23); a23 = o_sub(t265, a23); }
    { uint64_t t266 = a47; a47 = o_add(t266, a119); a119 = o_sub(t266, a119); }
    uint64_t t267 = a71;
    a71 = o_add(a71, a95);
    a95 = o_mul(a95, 4611686017353646080ULL);
    a47 = o_mul(a47, 16181989089180173841ULL);
    a23 = o_mul(a23, 5818851782451133869ULL);
    a119 = o_mul(a119, 11322249509082494407ULL);
    a95 = o_add(a95, t267);
    { uint64_t t268 = a95; a95 = o_add(t268, a23); a23 = o_sub(t268, a23); }
    { uint64_t t269 = a119; a119 = o_add(t269, a47); a47 = o_sub(t269, a47); }
    a47 = o_shift(a47, 48);
    { uint64_t t270 = a95; a95 = o_add(t270, a119); a119 = o_sub(t270, a119); }
    { uint64_t t271 = a23; a23 = o_add(t271, a47); a47 = o_sub(t271, a47); }
    { uint64_t t272 = a11; a11 = o_add(t272, a71); a71 = o_sub(t272, a71); }
    { uint64_t t273 = a35; a35 = o_add(t273, a95); a95 = o_sub(t273, a95); }
    { uint64_t t274 = a83; a83 = o_add(t274, a23); a23 = o_sub(t274, a23); }
    { uint64_t t275 = a107; a107 = o_add(t275, a47); a47 = o_sub(t275, a47); }
    { uint64_t t276 = a59; a59 = o_add(t276, a119); a119 = o_sub(t276, a119); }
    a85 = o_mul(a85, 12342513394488208227ULL);
    a73 = o_mul(a73, 5927015354646419725ULL);
    a37 = o_mul(a37, 9148693690730647261ULL);
    a49 = o_mul(a49, 6868348408044855211ULL);
    a61 = o_shift(a61, 8);
    a25 = o_mul(a25, 5290193119087387221ULL);
    a13 = o_mul(a13, 4682917097487535278ULL);
    a97 = o_mul(a97, 17775832080808074370ULL);
    a109 = o_mul(a109, 5856505865097423521ULL);
    a86 = o_mul(a86, 5927015354646419725ULL);
    a74 = o_mul(a74, 6868348408044855211ULL);
    a38 = o_mul(a38, 5290193119087387221ULL);
    a50 = o_mul(a50, 17775832080808074370ULL);
    a62 = o_shift(a62, 16);
    a26 = o_mul(a26, 18235156514275634624ULL);
    a14 = o_mul(a14, 5079231842359091375ULL);
    a98 = o_mul(a98, 9988211933311186582ULL);
    a110 = o_mul(a110, 8149776168132872528ULL);
    a87 = o_mul(a87, 9148693690730647261ULL);
    a75 = o_mul(a75, 5290193119087387221ULL);
    a39 = o_mul(a39, 5856505865097423521ULL);
    a51 = o_mul(a51, 18235156514275634624ULL);
    a63 = o_shift(a63, 24);
    a27 = o_mul(a27, 8149776168132872528ULL);
    a15 = o_mul(a15, 11331573348451128694ULL);
    a99 = o_mul(a99, 1041288259238279555ULL);
    a111 = o_mul(a111, 4419751934697861046ULL);
    a88 = o_mul(a88, 6868348408044855211ULL);
    a76 = o_mul(a76, 17775832080808074370ULL);
    a40 = o_mul(a40, 18235156514275634624ULL);
    a52 = o_mul(a52, 9988211933311186582ULL);
    a64 = o_shift(a64, 32);
    a28 = o_mul(a28, 1041288259238279555ULL);
    a16 = o_mul(a16, 15149912995474149095ULL);
    a100 = o_mul(a100, 6205107048362784195ULL);
    a112 = o_mul(a112, 17073700798457888299ULL);
    a89 = o_shift(a89, 8);
    a77 = o_shift(a77, 16);
    a41 = o_shift(a41, 24);
    a53 = o_shift(a53, 32);
    a65 = o_shift(a65, 40);
    a29 = o_shift(a29, 48);
    a17 = o_shift(a17, 56);
    a101 = o_shift(a101, 64);
    a113 = o_shift(a113, 72);
    a90 = o_mul(a90, 5290193119087387221ULL);
    a78 = o_mul(a78, 18235156514275634624ULL);
    a42 = o_mul(a42, 8149776168132872528ULL);
    a54 = o_mul(a54, 1041288259238279555ULL);
    a66 = o_shift(a66, 48);
    a30 = o_mul(a30, 17073700798457888299ULL);
    a18 = o_mul(a18, 17869255328328231396ULL);
    a102 = o_mul(a102, 15820824984080659046ULL);
    a114 = o_mul(a114, 2281812832982421726ULL);
    a91 = o_mul(a91, 4682917097487535278ULL);
    a79 = o_mul(a79, 5079231842359091375ULL);
    a43 = o_mul(a43, 11331573348451128694ULL);
    a55 = o_mul(a55, 15149912995474149095ULL);
    a67 = o_shift(a67, 56);
    a31 = o_mul(a31, 17869255328328231396ULL);
    a19 = o_mul(a19, 2458871528097962065ULL);
    a103 = o_mul(a103, 7085488865146701717ULL);
    a115 = o_mul(a115, 9298050378683937060ULL);
    a92 = o_mul(a92, 17775832080808074370ULL);
    a80 = o_mul(a80, 9988211933311186582ULL);
    a44 = o_mul(a44, 1041288259238279555ULL);
    a56 = o_mul(a56, 6205107048362784195ULL);
    a68 = o_shift(a68, 64);
    a32 = o_mul(a32, 15820824984080659046ULL);
    a20 = o_mul(a20, 7085488865146701717ULL);
    a104 = o_mul(a104, 11578395661369729110ULL);
    a116 = o_mul(a116, 211587555138949697ULL);
    a93 = o_mul(a93, 5856505865097423521ULL);
    a81 = o_mul(a81, 8149776168132872528ULL);
    a45 = o_mul(a45, 4419751934697861046ULL);
    a57 = o_mul(a57, 17073700798457888299ULL);
    a69 = o_shift(a69, 72);
    a33 = o_mul(a33, 2281812832982421726ULL);
    a21 = o_mul(a21, 9298050378683937060ULL);
    a105 = o_mul(a105, 211587555138949697ULL);
    a117 = o_mul(a117, 7115170720963455627ULL);
    a94 = o_shift(a94, 16);
    a82 = o_shift(a82, 32);
    a46 = o_shift(a46, 48);
    a58 = o_shift(a58, 64);
    a70 = o_shift(a70, 80);
    a34 = o_neg(a34);
    a22 = o_neg(o_shift(a22, 16));
    a106 = o_neg(o_shift(a106, 32));
    a118 = o_neg(o_shift(a118, 48));
    a95 = o_mul(a95, 7677121419106473143ULL);
    a83 = o_mul(a83, 5349526613560066800ULL);
    a47 = o_mul(a47, 4561472264319460910ULL);
    a59 = o_mul(a59, 12619683920608008665ULL);
    a71 = o_shift(a71, 88);
    a35 = o_mul(a35, 13156550950327197100ULL);
    a23 = o_mul(a23, 17272925976741953790ULL);
    a107 = o_mul(a107, 3296831073940435226ULL);
    a119 = o_mul(a119, 15587202262274831207ULL);
    { uint64_t t277 = a0; a0 = o_add(t277, a6); a6 = o_sub(t277, a6); }
    { uint64_t t278 = a3; a3 = o_add(t278, a9); a9 = o_sub(t278, a9); }
    a9 = o_shift(a9, 48);
    { uint64_t t279 = a0; a0 = o_add(t279, a3); a3 = o_sub(t279, a3); }
    { uint64_t t280 = a6; a6 = o_add(t280, a9); a9 = o_sub(t280, a9); }
    { uint64_t t281 = a4; a4 = o_add(t281, a10); a10 = o_sub(t281, a10); }
    { uint64_t t282 = a7; a7 = o_add(t282, a1); a1 = o_sub(t282, a1); }
    a1 = o_shift(a1, 48);
    { uint64_t t283 = a4; a4 = o_add(t283, a7); a7 = o_sub(t283, a7); }
    { uint64_t t284 = a10; a10 = o_add(t284, a1); a1 = o_sub(t284, a1); }
    { uint64_t t285 = a8; a8 = o_add(t285, a2); a2 = o_sub(t285, a2); }
    { uint64_t t286 = a11; a11 = o_add(t286, a5); a5 = o_sub(t286, a5); }
    a5 = o_shift(a5, 48);
    { uint64_t t287 = a8; a8 = o_add(t287, a11); a11 = o_sub(t287, a11); }
    { uint64_t t288 = a2; a2 = o_add(t288, a5); a5 = o_sub(t288, a5); }
    { uint64_t t289 = a0, t290 = a4, t291 = a8;
      a0 = o_add(o_add(t289, t290), t291);
      a4 = o_sub(o_add(t289, o_shift(t290, 64)), o_shift(t291, 32));
      a8 = o_add(o_sub(t289, o_shift(t290, 32)), o_shift(t291, 64)); }
    { uint64_t t292 = a6, t293 = a10, t294 = a2;
      a6 = o_add(o_add(t292, t293), t294);
      a10 = o_sub(o_add(t292, o_shift(t293, 64)), o_shift(t294, 32));
      a2 = o_add(o_sub(t292, o_shift(t293, 32)), o_shift(t294, 64)); }
    { uint64_t t295 = a3, t296 = a7, t297 = a11;
      a3 = o_add(o_add(t295, t296), t297);
      a7 = o_sub(o_add(t295, o_shift(t296, 64)), o_shift(t297, 32));
      a11 = o_add(o_sub(t295, o_shift(t296, 32)), o_shift(t297, 64)); }
    { uint64_t t298 = a9, t299 = a1, t300 = a5;
      a9 = o_add(o_add(t298, t299), t300);
      a1 = o_sub(o_add(t298, o_shift(t299, 64)), o_shift(t300, 32));
      a5 = o_add(o_sub(t298, o_shift(t299, 32)), o_shift(t300, 64)); }
    { uint64_t t301 = a84; a84 = o_add(t301, a90); a90 = o_sub(t301, a90); }
    { uint64_t t302 = a87; a87 = o_add(t302, a93); a93 = o_sub(t302, a93); }
    a93 = o_shift(a93, 48);
    { uint64_t t303 = a84; a84 = o_add(t303, a87); a87 = o_sub(t303, a87); }
    { uint64_t t304 = a90; a90 = o_add(t304, a93); a93 = o_sub(t304, a93); }
    { uint64_t t305 = a88; a88 = o_add(t305, a94); a94 = o_sub(t305, a94); }
    { uint64_t t306 = a91; a91 = o_add(t306, a85); a85 = o_sub(t306, a85); }
    a85 = o_shift(a85, 48);
    { uint64_t t307 = a88; a88 = o_add(t307, a91); a91 = o_sub(t307, a91); }
    { uint64_t t308 = a94; a94 = o_add(t308, a85); a85 = o_sub(t308, a85); }
    { uint64_t t309 = a92; a92 = o_add(t309, a86); a86 = o_sub(t309, a86); }
    { uint64_t t310 = a95; a95 = o_add(t310, a89); a89 = o_sub(t310, a89); }
    a89 = o_shift(a89, 48);
    { uint64_t t311 = a92; a92 = o_add(t311, a95); a95 = o_sub(t311, a95); }
    { uint64_t t312 = a86; a86 = o_add(t312, a89); a89 = o_sub(t312, a89); }
    { uint64_t t313 = a84, t314 = a88, t315 = a92;
      a84 = o_add(o_add(t313, t314), t315);
      a88 = o_sub(o_add(t313, o_shift(t314, 64)), o_shift(t315, 32));
      a92 = o_add(o_sub(t313, o_shift(t314, 32)), o_shift(t315, 64)); }
    { uint64_t t316 = a90, t317 = a94, t318 = a86;
      a90 = o_add(o_add(t316, t317), t318);
      a94 = o_sub(o_add(t316, o_shift(t317, 64)), o_shift(t318, 32));
      a86 = o_add(o_sub(t316, o_shift(t317, 32)), o_shift(t318, 64)); }
    { uint64_t t319 = a87, t320 = a91, t321 = a95;
      a87 = o_add(o_add(t319, t320), t321);
      a91 = o_sub(o_add(t319, o_shift(t320, 64)), o_shift(t321, 32));
      a95 = o_add(o_sub(t319, o_shift(t320, 32)), o_shift(t321, 64)); }
    { uint64_t t322 = a93, t323 = a85, t324 = a89;
      a93 = o_add(o_add(t322, t323), t324);
      a85 = o_sub(o_add(t322, o_shift(t323, 64)), o_shift(t324, 32));
      a89 = o_add(o_sub(t322, o_shift(t323, 32)), o_shift(t324, 64)); }
    { uint64_t t325 = a72; a72 = o_add(t325, a78); a78 = o_sub(t325, a78); }
    { uint64_t t326 = a75; a75 = o_add(t326, a81); a81 = o_sub(t326, a81); }
    a81 = o_shift(a81, 48);
    { uint64_t t327 = a72; a72 = o_add(t327, a75); a75 = o_sub(t327, a75); }
    { uint64_t t328 = a78; a78 = o_add(t328, a81); a81 = o_sub(t328, a81); }
    { uint64_t t329 = a76; a76 = o_add(t329, a82); a82 = o_sub(t329, a82); }
    { uint64_t t330 = a79; a79 = o_add(t330, a73); a73 = o_sub(t330, a73); }
    a73 = o_shift(a73, 48);
    { uint64_t t331 = a76; a76 = o_add(t331, a79); a79 = o_sub(t331, a79); }
    { uint64_t t332 = a82; a82 = o_add(t332, a73); a73 = o_sub(t332, a73); }
    { uint64_t t333 = a80; a80 = o_add(t333, a74); a74 = o_sub(t333, a74); }
    { uint64_t t334 = a83; a83 = o_add(t334, a77); a77 = o_sub(t334, a77); }
    a77 = o_shift(a77, 48);
    { uint64_t t335 = a80; a80 = o_add(t335, a83); a83 = o_sub(t335, a83); }
    { uint64_t t336 = a74; a74 = o_add(t336, a77); a77 = o_sub(t336, a77); }
    { uint64_t t337 = a72, t338 = a76, t339 = a80;
      a72 = o_add(o_add(t337, t338), t339);
      a76 = o_sub(o_add(t337, o_shift(t338, 64)), o_shift(t339, 32));
      a80 = o_add(o_sub(t337, o_shift(t338, 32)), o_shift(t339, 64)); }
    { uint64_t t340 = a78, t341 = a82, t342 = a74;
      a78 = o_add(o_add(t340, t341), t342);
      a82 = o_sub(o_add(t340, o_shift(t341, 64)), o_shift(t342, 32));
      a74 = o_add(o_sub(t340, o_shift(t341, 32)), o_shift(t342, 64)); }
    { uint64_t t343 = a75, t344 = a79, t345 = a83;
      a75 = o_add(o_add(t343, t344), t345);
      a79 = o_sub(o_add(t343, o_shift(t344, 64)), o_shift(t345, 32));
      a83 = o_add(o_sub(t343, o_shift(t344, 32)), o_shift(t345, 64)); }
    { uint64_t t346 = a81, t347 = a73, t348 = a77;
      a81 = o_add(o_add(t346, t347), t348);
      a73 = o_sub(o_add(t346, o_shift(t347, 64)), o_shift(t348, 32));
      a77 = o_add(o_sub(t346, o_shift(t347, 32)), o_shift(t348, 64)); }
    { uint64_t t349 = a36; a36 = o_add(t349, a42); a42 = o_sub(t349, a42); }
    { uint64_t t350 = a39; a39 = o_add(t350, a45); a45 = o_sub(t350, a45); }
    a45 = o_shift(a45, 48);
    { uint64_t t351 = a36; a36 = o_add(t351, a39); a39 = o_sub(t351, a39); }
    { uint64_t t352 = a42; a42 = o_add(t352, a45); a45 = o_sub(t352, a45); }
    { uint64_t t353 = a40; a40 = o_add(t353, a46); a46 = o_sub(t353, a46); }
    { uint64_t t354 = a43; a43 = o_add(t354, a37); a37 = o_sub(t354, a37); }
    a37 = o_shift(a37, 48);
    { uint64_t t355 = a40; a40 = o_add(t355, a43); a43 = o_sub(t355, a43); }
    { uint64_t t356 = a46; a46 = o_add(t356, a37); a37 = o_sub(t356, a37); }
    { uint64_t t357 = a44; a44 = o_add(t357, a38); a38 = o_sub(t357, a38); }
    { uint64_t t358 = a47; a47 = o_add(t358, a41); a41 = o_sub(t358, a41); }
    a41 = o_shift(a41, 48);
    { uint64_t t359 = a44; a44 = o_add(t359, a47); a47 = o_sub(t359, a47); }
    { uint64_t t360 = a38; a38 = o_add(t360, a41); a41 = o_sub(t360, a41); }
    { uint64_t t361 = a36, t362 = a40, t363 = a44;
      a36 = o_add(o_add(t361, t362), t363);
      a40 = o_sub(o_add(t361, o_shift(t362, 64)), o_shift(t363, 32));
      a44 = o_add(o_sub(t361, o_shift(t362, 32)), o_shift(t363, 64)); }
    { uint64_t t364 = a42, t365 = a46, t366 = a38;
      a42 = o_add(o_add(t364, t365), t366);
      a46 = o_sub(o_add(t364, o_shift(t365, 64)), o_shift(t366, 32));
      a38 = o_add(o_sub(t364, o_shift(t365, 32)), o_shift(t366, 64)); }
    { uint64_t t367 = a39, t368 = a43, t369 = a47;
      a39 = o_add(o_add(t367, t368), t369);
      a43 = o_sub(o_add(t367, o_shift(t368, 64)), o_shift(t369, 32));
      a47 = o_add(o_sub(t367, o_shift(t368, 32)), o_shift(t369, 64)); }
    { uint64_t t370 = a45, t371 = a37, t372 = a41;
      a45 = o_add(o_add(t370, t371), t372);
      a37 = o_sub(o_add(t370, o_shift(t371, 64)), o_shift(t372, 32));
      a41 = o_add(o_sub(t370, o_shift(t371, 32)), o_shift(t372, 64)); }
    { uint64_t t373 = a48; a48 = o_add(t373, a54); a54 = o_sub(t373, a54); }
    { uint64_t t374 = a51; a51 = o_add(t374, a57); a57 = o_sub(t374, a57); }
    a57 = o_shift(a57, 48);
    { uint64_t t375 = a48; a48 = o_add(t375, a51); a51 = o_sub(t375, a51); }
    { uint64_t t376 = a54; a54 = o_add(t376, a57); a57 = o_sub(t376, a57); }
    { uint64_t t377 = a52; a52 = o_add(t377, a58); a58 = o_sub(t377, a58); }
    { uint64_t t378 = a55; a55 = o_add(t378, a49); a49 = o_sub(t378, a49); }
    a49 = o_shift(a49, 48);
    { uint64_t t379 = a52; a52 = o_add(t379, a55); a55 = o_sub(t379, a55); }
    { uint64_t t380 = a58; a58 = o_add(t380, a49); a49 = o_sub(t380, a49); }
    { uint64_t t381 = a56; a56 = o_add(t381, a50); a50 = o_sub(t381, a50); }
    { uint64_t t382 = a59; a59 = o_add(t382, a53); a53 = o_sub(t382, a53); }
    a53 = o_shift(a53, 48);
    { uint64_t t383 = a56; a56 = o_add(t383, a59); a59 = o_sub(t383, a59); }
    { uint64_t t384 = a50; a50 = o_add(t384, a53); a53 = o_sub(t384, a53); }
    { uint64_t t385 = a48, t386 = a52, t387 = a56;
      a48 = o_add(o_add(t385, t386), t387);
      a52 = o_sub(o_add(t385, o_shift(t386, 64)), o_shift(t387, 32));
      a56 = o_add(o_sub(t385, o_shift(t386, 32)), o_shift(t387, 64)); }
    { uint64_t t388 = a54, t389 = a58, t390 = a50;
      a54 = o_add(o_add(t388, t389), t390);
      a58 = o_sub(o_add(t388, o_shift(t389, 64)), o_shift(t390, 32));
      a50 = o_add(o_sub(t388, o_shift(t389, 32)), o_shift(t390, 64)); }
    { uint64_t t391 = a51, t392 = a55, t393 = a59;
      a51 = o_add(o_add(t391, t392), t393);
      a55 = o_sub(o_add(t391, o_shift(t392, 64)), o_shift(t393, 32));
      a59 = o_add(o_sub(t391, o_shift(t392, 32)), o_shift(t393, 64)); }
    { uint64_t t394 = a57, t395 = a49, t396 = a53;
      a57 = o_add(o_add(t394, t395), t396);
      a49 = o_sub(o_add(t394, o_shift(t395, 64)), o_shift(t396, 32));
      a53 = o_add(o_sub(t394, o_shift(t395, 32)), o_shift(t396, 64)); }
    { uint64_t t397 = a60; a60 = o_add(t397, a66); a66 = o_sub(t397, a66); }
    { uint64_t t398 = a63; a63 = o_add(t398, a69); a69 = o_sub(t398, a69); }
    a69 = o_shift(a69, 48);
    { uint64_t t399 = a60; a60 = o_add(t399, a63); a63 = o_sub(t399, a63); }
    { uint64_t t400 = a66; a66 = o_add(t400, a69); a69 = o_sub(t400, a69); }
    { uint64_t t401 = a64; a64 = o_add(t401, a70); a70 = o_sub(t401, a70); }
    { uint64_t t402 = a67; a67 = o_add(t402, a61); a61 = o_sub(t402, a61); }
    a61 = o_shift(a61, 48);
    { uint64_t t403 = a64; a64 = o_add(t403, a67); a67 = o_sub(t403, a67); }
    { uint64_t t404 = a70; a70 = o_add(t404, a61); a61 = o_sub(t404, a61); }
    { uint64_t t405 = a68; a68 = o_add(t405, a62); a62 = o_sub(t405, a62); }
    { uint64_t t406 = a71; a71 = o_add(t406, a65); a65 = o_sub(t406, a65); }
    a65 = o_shift(a65, 48);
    { uint64_t t407 = a68; a68 = o_add(t407, a71); a71 = o_sub(t407, a71); }
    { uint64_t t408 = a62; a62 = o_add(t408, a65); a65 = o_sub(t408, a65); }
    { uint64_t t409 = a60, t410 = a64, t411 = a68;
      a60 = o_add(o_add(t409, t410), t411);
      a64 = o_sub(o_add(t409, o_shift(t410, 64)), o_shift(t411, 32));
      a68 = o_add(o_sub(t409, o_shift(t410, 32)), o_shift(t411, 64)); }
    { uint64_t t412 = a66, t413 = a70, t414 = a62;
      a66 = o_add(o_add(t412, t413), t414);
      a70 = o_sub(o_add(t412, o_shift(t413, 64)), o_shift(t414, 32));
      a62 = o_add(o_sub(t412, o_shift(t413, 32)), o_shift(t414, 64)); }
    { uint64_t t415 = a63, t416 = a67, t417 = a71;
      a63 = o_add(o_add(t415, t416), t417);
      a67 = o_sub(o_add(t415, o_shift(t416, 64)), o_shift(t417, 32));
      a71 = o_add(o_sub(t415, o_shift(t416, 32)), o_shift(t417, 64)); }
    { uint64_t t418 = a69, t419 = a61, t420 = a65;
      a69 = o_add(o_add(t418, t419), t420);
      a61 = o_sub(o_add(t418, o_shift(t419, 64)), o_shift(t420, 32));
      a65 = o_add(o_sub(t418, o_shift(t419, 32)), o_shift(t420, 64)); }
    { uint64_t t421 = a24; a24 = o_add(t421, a30); a30 = o_sub(t421, a30); }
    { uint64_t t422 = a27; a27 = o_add(t422, a33); a33 = o_sub(t422, a33); }
    a33 = o_shift(a33, 48);
    { uint64_t t423 = a24; a24 = o_add(t423, a27); a27 = o_sub(t423, a27); }
    { uint64_t t424 = a30; a30 = o_add(t424, a33); a33 = o_sub(t424, a33); }
    { uint64_t t425 = a28; a28 = o_add(t425, a34); a34 = o_sub(t425, a34); }
    { uint64_t t426 = a31; a31 = o_add(t426, a25); a25 = o_sub(t426, a25); }
    a25 = o_shift(a25, 48);
    { uint64_t t427 = a28; a28 = o_add(t427, a31); a31 = o_sub(t427, a31); }
    { uint64_t t428 = a34; a34 = o_add(t428, a25); a25 = o_sub(t428, a25); }
    { uint64_t t429 = a32; a32 = o_add(t429, a26); a26 = o_sub(t429, a26); }
    { uint64_t t430 = a35; a35 = o_add(t430, a29); a29 = o_sub(t430, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t431 = a32; a32 = o_add(t431, a35); a35 = o_sub(t431, a35); }
    { uint64_t t432 = a26; a26 = o_add(t432, a29); a29 = o_sub(t432, a29); }
    { uint64_t t433 = a24, t434 = a28, t435 = a32;
      a24 = o_add(o_add(t433, t434), t435);
      a28 = o_sub(o_add(t433, o_shift(t434, 64)), o_shift(t435, 32));
      a32 = o_add(o_sub(t433, o_shift(t434, 32)), o_shift(t435, 64)); }
    { uint64_t t436 = a30, t437 = a34, t438 = a26;
      a30 = o_add(o_add(t436, t437), t438);
      a34 = o_sub(o_add(t436, o_shift(t437, 64)), o_shift(t438, 32));
      a26 = o_add(o_sub(t436, o_shift(t437, 32)), o_shift(t438, 64)); }
    { uint64_t t439 = a27, t440 = a31, t441 = a35;
      a27 = o_add(o_add(t439, t440), t441);
      a31 = o_sub(o_add(t439, o_shift(t440, 64)), o_shift(t441, 32));
      a35 = o_add(o_sub(t439, o_shift(t440, 32)), o_shift(t441, 64)); }
    { uint64_t t442 = a33, t443 = a25, t444 = a29;
      a33 = o_add(o_add(t442, t443), t444);
      a25 = o_sub(o_add(t442, o_shift(t443, 64)), o_shift(t444, 32));
      a29 = o_add(o_sub(t442, o_shift(t443, 32)), o_shift(t444, 64)); }
    { uint64_t t445 = a12; a12 = o_add(t445, a18); a18 = o_sub(t445, a18); }
    { uint64_t t446 = a15; a15 = o_add(t446, a21); a21 = o_sub(t446, a21); }
    a21 = o_shift(a21, 48);
    { uint64_t t447 = a12; a12 = o_add(t447, a15); a15 = o_sub(t447, a15); }
    { uint64_t t448 = a18; a18 = o_add(t448, a21); a21 = o_sub(t448, a21); }
    { uint64_t t449 = a16; a16 = o_add(t449, a22); a22 = o_sub(t449, a22); }
    { uint64_t t450 = a19; a19 = o_add(t450, a13); a13 = o_sub(t450, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t451 = a16; a16 = o_add(t451, a19); a19 = o_sub(t451, a19); }
    { uint64_t t452 = a22; a22 = o_add(t452, a13); a13 = o_sub(t452, a13); }
    { uint64_t t453 = a20; a20 = o_add(t453, a14); a14 = o_sub(t453, a14); }
    { uint64_t t454 = a23; a23 = o_add(t454, a17); a17 = o_sub(t454, a17); }
    a17 = o_shift(a17, 48);
    { uint64_t t455 = a20; a20 = o_add(t455, a23); a23 = o_sub(t455, a23); }
    { uint64_t t456 = a14; a14 = o_add(t456, a17); a17 = o_sub(t456, a17); }
    { uint64_t t457 = a12, t458 = a16, t459 = a20;
      a12 = o_add(o_add(t457, t458), t459);
      a16 = o_sub(o_add(t457, o_shift(t458, 64)), o_shift(t459, 32));
      a20 = o_add(o_sub(t457, o_shift(t458, 32)), o_shift(t459, 64)); }
    { uint64_t t460 = a18, t461 = a22, t462 = a14;
      a18 = o_add(o_add(t460, t461), t462);
      a22 = o_sub(o_add(t460, o_shift(t461, 64)), o_shift(t462, 32));
      a14 = o_add(o_sub(t460, o_shift(t461, 32)), o_shift(t462, 64)); }
    { uint64_t t463 = a15, t464 = a19, t465 = a23;
      a15 = o_add(o_add(t463, t464), t465);
      a19 = o_sub(o_add(t463, o_shift(t464, 64)), o_shift(t465, 32));
      a23 = o_add(o_sub(t463, o_shift(t464, 32)), o_shift(t465, 64)); }
    { uint64_t t466 = a21, t467 = a13, t468 = a17;
      a21 = o_add(o_add(t466, t467), t468);
      a13 = o_sub(o_add(t466, o_shift(t467, 64)), o_shift(t468, 32));
      a17 = o_add(o_sub(t466, o_shift(t467, 32)), o_shift(t468, 64)); }
    { uint64_t t469 = a96; a96 = o_add(t469, a102); a102 = o_sub(t469, a102); }
    { uint64_t t470 = a99; a99 = o_add(t470, a105); a105 = o_sub(t470, a105); }
    a105 = o_shift(a105, 48);
    { uint64_t t471 = a96; a96 = o_add(t471, a99); a99 = o_sub(t471, a99); }
    { uint64_t t472 = a102; a102 = o_add(t472, a105); a105 = o_sub(t472, a105); }
    { uint64_t t473 = a100; a100 = o_add(t473, a106); a106 = o_sub(t473, a106); }
    { uint64_t t474 = a103; a103 = o_add(t474, a97); a97 = o_sub(t474, a97); }
    a97 = o_shift(a97, 48);
    { uint64_t t475 = a100; a100 = o_add(t475, a103); a103 = o_sub(t475, a103); }
    { uint64_t t476 = a106; a106 = o_add(t476, a97); a97 = o_sub(t476, a97); }
    { uint64_t t477 = a104; a104 = o_add(t477, a98); a98 = o_sub(t477, a98); }
    { uint64_t t478 = a107; a107 = o_add(t478, a101); a101 = o_sub(t478, a101); }
    a101 = o_shift(a101, 48);
    { uint64_t t479 = a104; a104 = o_add(t479, a107); a107 = o_sub(t479, a107); }
    { uint64_t t480 = a98; a98 = o_add(t480, a101); a101 = o_sub(t480, a101); }
    { uint64_t t481 = a96, t482 = a100, t483 = a104;
      a96 = o_add(o_add(t481, t482), t483);
      a100 = o_sub(o_add(t481, o_shift(t482, 64)), o_shift(t483, 32));
      a104 = o_add(o_sub(t481, o_shift(t482, 32)), o_shift(t483, 64)); }
    { uint64_t t484 = a102, t485 = a106, t486 = a98;
      a102 = o_add(o_add(t484, t485), t486);
      a106 = o_sub(o_add(t484, o_shift(t485, 64)), o_shift(t486, 32));
      a98 = o_add(o_sub(t484, o_shift(t485, 32)), o_shift(t486, 64)); }
    { uint64_t t487 = a99, t488 = a103, t489 = a107;
      a99 = o_add(o_add(t487, t488), t489);
      a103 = o_sub(o_add(t487, o_shift(t488, 64)), o_shift(t489, 32));
      a107 = o_add(o_sub(t487, o_shift(t488, 32)), o_shift(t489, 64)); }
    { uint64_t t490 = a105, t491 = a97, t492 = a101;
      a105 = o_add(o_add(t490, t491), t492);
      a97 = o_sub(o_add(t490, o_shift(t491, 64)), o_shift(t492, 32));
      a101 = o_add(o_sub(t490, o_shift(t491, 32)), o_shift(t492, 64)); }
    { uint64_t t493 = a108; a108 = o_add(t493, a114); a114 = o_sub(t493, a114); }
    { uint64_t t494 = a111; a111 = o_add(t494, a117); a117 = o_sub(t494, a117); }
    a117 = o_shift(a117, 48);
    { uint64_t t495 = a108; a108 = o_add(t495, a111); a111 = o_sub(t495, a111); }
    { uint64_t t496 = a114; a114 = o_add(t496, a117); a117 = o_sub(t496, a117); }
    { uint64_t t497 = a112; a112 = o_add(t497, a118); a118 = o_sub(t497, a118); }
    { uint64_t t498 = a115; a115 = o_add(t498, a109); a109 = o_sub(t498, a109); }
    a109 = o_shift(a109, 48);
    { uint64_t t499 = a112; a112 = o_add(t499, a115); a115 = o_sub(t499, a115); }
    { uint64_t t500 = a118; a118 = o_add(t500, a109); a109 = o_sub(t500, a109); }
    { uint64_t t501 = a116; a116 = o_add(t501, a110); a110 = o_sub(t501, a110); }
    { uint64_t t502 = a119; a119 = o_add(t502, a113); a113 = o_sub(t502, a113); }
    a113 = o_shift(a113, 48);
    { uint64_t t503 = a116; a116 = o_add(t503, a119); a119 = o_sub(t503, a119); }
    { uint64_t t504 = a110; a110 = o_add(t504, a113); a113 = o_sub(t504, a113); }
    { uint64_t t505 = a108, t506 = a112, t507 = a116;
      a108 = o_add(o_add(t505, t506), t507);
      a112 = o_sub(o_add(t505, o_shift(t506, 64)), o_shift(t507, 32));
      a116 = o_add(o_sub(t505, o_shift(t506, 32)), o_shift(t507, 64)); }
    { uint64_t t508 = a114, t509 = a118, t510 = a110;
      a114 = o_add(o_add(t508, t509), t510);
      a118 = o_sub(o_add(t508, o_shift(t509, 64)), o_shift(t510, 32));
      a110 = o_add(o_sub(t508, o_shift(t509, 32)), o_shift(t510, 64)); }
    { uint64_t t511 = a111, t512 = a115, t513 = a119;
      a111 = o_add(o_add(t511, t512), t513);
      a115 = o_sub(o_add(t511, o_shift(t512, 64)), o_shift(t513, 32));
      a119 = o_add(o_sub(t511, o_shift(t512, 32)), o_shift(t513, 64)); }
    { uint64_t t514 = a117, t515 = a109, t516 = a113;
      a117 = o_add(o_add(t514, t515), t516);
      a109 = o_sub(o_add(t514, o_shift(t515, 64)), o_shift(t516, 32));
      a113 = o_add(o_sub(t514, o_shift(t515, 32)), o_shift(t516, 64)); }
    v[0] = a0;
    v[1] = a84;
    v[2] = a72;
    v[3] = a36;
    v[4] = a48;
    v[5] = a60;
    v[6] = a24;
    v[7] = a12;
    v[8] = a96;
    v[9] = a108;
    v[10] = a10;
    v[11] = a94;
    v[12] = a82;
    v[13] = a46;
    v[14] = a58;
    v[15] = a70;
    v[16] = a34;
    v[17] = a22;
    v[18] = a106;
    v[19] = a118;
    v[20] = a11;
    v[21] = a95;
    v[22] = a83;
    v[23] = a47;
    v[24] = a59;
    v[25] = a71;
    v[26] = a35;
    v[27] = a23;
    v[28] = a107;
    v[29] = a119;
    v[30] = a9;
    v[31] = a93;
    v[32] = a81;
    v[33] = a45;
    v[34] = a57;
    v[35] = a69;
    v[36] = a33;
    v[37] = a21;
    v[38] = a105;
    v[39] = a117;
    v[40] = a4;
    v[41] = a88;
    v[42] = a76;
    v[43] = a40;
    v[44] = a52;
    v[45] = a64;
    v[46] = a28;
    v[47] = a16;
    v[48] = a100;
    v[49] = a112;
    v[50] = a2;
    v[51] = a86;
    v[52] = a74;
    v[53] = a38;
    v[54] = a50;
    v[55] = a62;
    v[56] = a26;
    v[57] = a14;
    v[58] = a98;
    v[59] = a110;
    v[60] = a3;
    v[61] = a87;
    v[62] = a75;
    v[63] = a39;
    v[64] = a51;
    v[65] = a63;
    v[66] = a27;
    v[67] = a15;
    v[68] = a99;
    v[69] = a111;
    v[70] = a1;
    v[71] = a85;
    v[72] = a73;
    v[73] = a37;
    v[74] = a49;
    v[75] = a61;
    v[76] = a25;
    v[77] = a13;
    v[78] = a97;
    v[79] = a109;
    v[80] = a8;
    v[81] = a92;
    v[82] = a80;
    v[83] = a44;
    v[84] = a56;
    v[85] = a68;
    v[86] = a32;
    v[87] = a20;
    v[88] = a104;
    v[89] = a116;
    v[90] = a6;
    v[91] = a90;
    v[92] = a78;
    v[93] = a42;
    v[94] = a54;
    v[95] = a66;
    v[96] = a30;
    v[97] = a18;
    v[98] = a102;
    v[99] = a114;
    v[100] = a7;
    v[101] = a91;
    v[102] = a79;
    v[103] = a43;
    v[104] = a55;
    v[105] = a67;
    v[106] = a31;
    v[107] = a19;
    v[108] = a103;
    v[109] = a115;
    v[110] = a5;
    v[111] = a89;
    v[112] = a77;
    v[113] = a41;
    v[114] = a53;
    v[115] = a65;
    v[116] = a29;
    v[117] = a17;
    v[118] = a101;
    v[119] = a113;
}

static void o_ntt_128(uint64_t *v) {
    uint64_t a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3], a4 = v[4], a5 = v[5], a6 = v[6], a7 = v[7], a8 = v[8], a9 = v[9], a10 = v[10], a11 = v[11], a12 = v[12], a13 = v[13], a14 = v[14], a15 = v[15], a16 = v[16], a17 = v[17], a18 = v[18], a19 = v[19], a20 = v[20], a21 = v[21], a22 = v[22], a23 = v[23], a24 = v[24], a25 = v[25], a26 = v[26], a27 = v[27], a28 = v[28], a29 = v[29], a30 = v[30], a31 = v[31], a32 = v[32], a33 = v[33], a34 = v[34], a35 = v[35], a36 = v[36], a37 = v[37], a38 = v[38], a39 = v[39], a40 = v[40], a41 = v[41], a42 = v[42], a43 = v[43], a44 = v[44], a45 = v[45], a46 = v[46], a47 = v[47], a48 = v[48], a49 = v[49], a50 = v[50], a51 = v[51], a52 = v[52], a53 = v[53], a54 = v[54], a55 = v[55], a56 = v[56], a57 = v[57], a58 = v[58], a59 = v[59], a60 = v[60], a61 = v[61], a62 = v[62], a63 = v[63], a64 = v[64], a65 = v[65], a66 = v[66], a67 = v[67], a68 = v[68], a69 = v[69], a70 = v[70], a71 = v[71], a72 = v[72], a73 = v[73], a74 = v[74], a75 = v[75], a76 = v[76], a77 = v[77], a78 = v[78], a79 = v[79], a80 = v[80], a81 = v[81], a82 = v[82], a83 = v[83], a84 = v[84], a85 = v[85], a86 = v[86], a87 = v[87], a88 = v[88], a89 = v[89], a90 = v[90], a91 = v[91], a92 = v[92], a93 = v[93], a94 = v[94], a95 = v[95], a96 = v[96], a97 = v[97], a98 = v[98], a99 = v[99], a100 = v[100], a101 = v[101], a102 = v[102], a103 = v[103], a104 = v[104], a105 = v[105], a106 = v[106], a107 = v[107], a108 = v[108], a109 = v[109], a110 = v[110], a111 = v[111], a112 = v[112], a113 = v[113], a114 = v[114], a115 = v[115], a116 = v[116], a117 = v[117], a118 = v[118], a119 = v[119], a120 = v[120], a121 = v[121], a122 = v[122], a123 = v[123], a124 = v[124], a125 = v[125], a126 = v[126], a127 = v[127];
    { uint64_t t1 = a0; a0 = o_add(t1, a64); a64 = o_sub(t1, a64); }
    { uint64_t t2 = a16; a16 = o_add(t2, a80); a80 = o_sub(t2, a80); }
    { uint64_t t3 = a32; a32 = o_add(t3, a96); a96 = o_sub(t3, a96); }
    { uint64_t t4 = a48; a48 = o_add(t4, a112); a112 = o_sub(t4, a112); }
    a80 = o_shift(a80, 24);
    a96 = o_shift(a96, 48);
    a112 = o_shift(a112, 72);
    { uint64_t t5 = a0; a0 = o_add(t5, a32); a32 = o_sub(t5, a32); }
    { uint64_t t6 = a16; a16 = o_add(t6, a48); a48 = o_sub(t6, a48); }
    a48 = o_shift(a48, 48);
    { uint64_t t7 = a0; a0 = o_add(t7, a16); a16 = o_sub(t7, a16); }
    { uint64_t t8 = a32; a32 = o_add(t8, a48); a48 = o_sub(t8, a48); }
    { uint64_t t9 = a64; a64 = o_add(t9, a96); a96 = o_sub(t9, a96); }
    { uint64_t t10 = a80; a80 = o_add(t10, a112); a112 = o_sub(t10, a112); }
    a112 = o_shift(a112, 48);
    { uint64_t t11 = a64; a64 = o_add(t11, a80); a80 = o_sub(t11, a80); }
    { uint64_t t12 = a96; a96 = o_add(t12, a112); a112 = o_sub(t12, a112); }
    { uint64_t t13 = a1; a1 = o_add(t13, a65); a65 = o_sub(t13, a65); }
    { uint64_t t14 = a17; a17 = o_add(t14, a81); a81 = o_sub(t14, a81); }
    { uint64_t t15 = a33; a33 = o_add(t15, a97); a97 = o_sub(t15, a97); }
    { uint64_t t16 = a49; a49 = o_add(t16, a113); a113 = o_sub(t16, a113); }
    a81 = o_shift(a81, 24);
    a97 = o_shift(a97, 48);
    a113 = o_shift(a113, 72);
    { uint64_t t17 = a1; a1 = o_add(t17, a33); a33 = o_sub(t17, a33); }
    { uint64_t t18 = a17; a17 = o_add(t18, a49); a49 = o_sub(t18, a49); }
    a49 = o_shift(a49, 48);
    { uint64_t t19 = a1; a1 = o_add(t19, a17); a17 = o_sub(t19, a17); }
    { uint64_t t20 = a33; a33 = o_add(t20, a49); a49 = o_sub(t20, a49); }
    { uint64_t t21 = a65; a65 = o_add(t21, a97); a97 = o_sub(t21, a97); }
    { uint64_t t22 = a81; a81 = o_add(t22, a113); a113 = o_sub(t22, a113); }
    a113 = o_shift(a113, 48);
    { uint64_t t23 = a65; a65 = o_add(t23, a81); a81 = o_sub(t23, a81); }
    { uint64_t t24 = a97; a97 = o_add(t24, a113); a113 = o_sub(t24, a113); }
    { uint64_t t25 = a2; a2 = o_add(t25, a66); a66 = o_sub(t25, a66); }
    { uint64_t t26 = a18; a18 = o_add(t26, a82); a82 = o_sub(t26, a82); }
    { uint64_t t27 = a34; a34 = o_add(t27, a98); a98 = o_sub(t27, a98); }
    { uint64_t t28 = a50; a50 = o_add(t28, a114); a114 = o_sub(t28, a114); }
    a82 = o_shift(a82, 24);
    a98 = o_shift(a98, 48);
    a114 = o_shift(a114, 72);
    { uint64_t t29 = a2; a2 = o_add(t29, a34); a34 = o_sub(t29, a34); }
    { uint64_t t30 = a18; a18 = o_add(t30, a50); a50 = o_sub(t30, a50); }
    a50 = o_shift(a50, 48);
    { uint64_t t31 = a2; a2 = o_add(t31, a18); a18 = o_sub(t31, a18); }
    { uint64_t t32 = a34; a34 = o_add(t32, a50); a50 = o_sub(t32, a50); }
    { uint64_t t33 = a66; a66 = o_add(t33, a98); a98 = o_sub(t33, a98); }
    { uint64_t t34 = a82; a82 = o_add(t34, a114); a114 = o_sub(t34, a114); }
    a114 = o_shift(a114, 48);
    { uint64_t t35 = a66; a66 = o_add(t35, a82); a82 = o_sub(t35, a82); }
    { uint64_t t36 = a98; a98 = o_add(t36, a114); a114 = o_sub(t36, a114); }
    { uint64_t t37 = a3; a3 = o_add(t37, a67); a67 = o_sub(t37, a67); }
    { uint64_t t38 = a19; a19 = o_add(t38, a83); a83 = o_sub(t38, a83); }
    { uint64_t t39 = a35; a35 = o_add(t39, a99); a99 = o_sub(t39, a99); }
    { uint64_t t40 = a51; a51 = o_add(t40, a115); a115 = o_sub(t40, a115); }
    a83 = o_shift(a83, 24);
    a99 = o_shift(a99, 48);
    a115 = o_shift(a115, 72);
    { uint64_t t41 = a3; a3 = o_add(t41, a35); a35 = o_sub(t41, a35); }
    { uint64_t t42 = a19; a19 = o_add(t42, a51); a51 = o_sub(t42, a51); }
    a51 = o_shift(a51, 48);
    { uint64_t t43 = a3; a3 = o_add(t43, a19); a19 = o_sub(t43, a19); }
    { uint64_t t44 = a35; a35 = o_add(t44, a51); a51 = o_sub(t44, a51); }
    { uint64_t t45 = a67; a67 = o_add(t45, a99); a99 = o_sub(t45, a99); }
    { uint64_t t46 = a83; a83 = o_add(t46, a115); a115 = o_sub(t46, a115); }
    a115 = o_shift(a115, 48);
    { uint64_t t47 = a67; a67 = o_add(t47, a83); a83 = o_sub(t47, a83); }
    { uint64_t t48 = a99; a99 = o_add(t48, a115); a115 = o_sub(t48, a115); }
    { uint64_t t49 = a4; a4 = o_add(t49, a68); a68 = o_sub(t49, a68); }
    { uint64_t t50 = a20; a20 = o_add(t50, a84); a84 = o_sub(t50, a84); }
    { uint64_t t51 = a36; a36 = o_add(t51, a100); a100 = o_sub(t51, a100); }
    { uint64_t t52 = a52; a52 = o_add(t52, a116); a116 = o_sub(t52, a116); }
    a84 = o_shift(a84, 24);
    a100 = o_shift(a100, 48);
    a116 = o_shift(a116, 72);
    { uint64_t t53 = a4; a4 = o_add(t53, a36); a36 = o_sub(t53, a36); }
    { uint64_t t54 = a20; a20 = o_add(t54, a52); a52 = o_sub(t54, a52); }
    a52 = o_shift(a52, 48);
    { uint64_t t55 = a4; a4 = o_add(t55, a20); a20 = o_sub(t55, a20); }
    { uint64_t t56 = a36; a36 = o_add(t56, a52); a52 = o_sub(t56, a52); }
    { uint64_t t57 = a68; a68 = o_add(t57, a100); a100 = o_sub(t57, a100); }
    { uint64_t t58 = a84; a84 = o_add(t58, a116); a116 = o_sub(t58, a116); }
    a116 = o_shift(a116, 48);
    { uint64_t t59 = a68; a68 = o_add(t59, a84); a84 = o_sub(t59, a84); }
    { uint64_t t60 = a100; a100 = o_add(t60, a116); a116 = o_sub(t60, a116); }
    { uint64_t t61 = a5; a5 = o_add(t61, a69); a69 = o_sub(t61, a69); }
    { uint64_t t62 = a21; a21 = o_add(t62, a85); a85 = o_sub(t62, a85); }
    { uint64_t t63 = a37; a37 = o_add(t63, a101); a101 = o_sub(t63, a101); }
    { uint64_t t64 = a53; a53 = o_add(t64, a117); a117 = o_sub(t64, a117); }
    a85 = o_shift(a85, 24);
    a101 = o_shift(a101, 48);
    a117 = o_shift(a117, 72);
    { uint64_t t65 = a5; a5 = o_add(t65, a37); a37 = o_sub(t65, a37); }
    { uint64_t t66 = a21; a21 = o_add(t66, a53); a53 = o_sub(t66, a53); }
    a53 = o_shift(a53, 48);
    { uint64_t t67 = a5; a5 = o_add(t67, a21); a21 = o_sub(t67, a21); }
    { uint64_t t68 = a37; a37 = o_add(t68, a53); a53 = o_sub(t68, a53); }
    { uint64_t t69 = a69; a69 = o_add(t69, a101); a101 = o_sub(t69, a101); }
    { uint64_t t70 = a85; a85 = o_add(t70, a117); a117 = o_sub(t70, a117); }
    a117 = o_shift(a117, 48);
    { uint64_t t71 = a69; a69 = o_add(t71, a85); a85 = o_sub(t71, a85); }
    { uint64_t t72 = a101; a101 = o_add(t72, a117); a117 = o_sub(t72, a117); }
    { uint64_t t73 = a6; a6 = o_add(t73, a70); a70 = o_sub(t73, a70); }
    { uint64_t t74 = a22; a22 = o_add(t74, a86); a86 = o_sub(t74, a86); }
    { uint64_t t75 = a38; a38 = o_add(t75, a102); a102 = o_sub(t75, a102); }
    { uint64_t t76 = a54; a54 = o_add(t76, a118); a118 = o_sub(t76, a118); }
    a86 = o_shift(a86, 24);
    a102 = o_shift(a102, 48);
    a118 = o_shift(a118, 72);
    { uint64_t t77 = a6; a6 = o_add(t77, a38); a38 = o_sub(t77, a38); }
    { uint64_t t78 = a22; a22 = o_add(t78, a54); a54 = o_sub(t78, a54); }
    a54 = o_shift(a54, 48);
    { uint64_t t79 = a6; a6 = o_add(t79, a22); a22 = o_sub(t79, a22); }
    { uint64_t t80 = a38; a38 = o_add(t80, a54); a54 = o_sub(t80, a54); }
    { uint64_t t81 = a70; a70 = o_add(t81, a102); a102 = o_sub(t81, a102); }
    { uint64_t t82 = a86; a86 = o_add(t82, a118); a118 = o_sub(t82, a118); }
    a118 = o_shift(a118, 48);
    { uint64_t t83 = a70; a70 = o_add(t83, a86); a86 = o_sub(t83, a86); }
    { uint64_t t84 = a102; a102 = o_add(t84, a118); a118 = o_sub(t84, a118); }
    { uint64_t t85 = a7; a7 = o_add(t85, a71); a71 = o_sub(t85, a71); }
    { uint64_t t86 = a23; a23 = o_add(t86, a87); a87 = o_sub(t86, a87); }
    { uint64_t t87 = a39; a39 = o_add(t87, a103); a103 = o_sub(t87, a103); }
    { uint64_t t88 = a55; a55 = o_add(t88, a119); a119 = o_sub(t88, a119); }
    a87 = o_shift(a87, 24);
    a103 = o_shift(a103, 48);
    a119 = o_shift(a119, 72);
    { uint64_t t89 = a7; a7 = o_add(t89, a39); a39 = o_sub(t89, a39); }
    { uint64_t t90 = a23; a23 = o_add(t90, a55); a55 = o_sub(t90, a55); }
    a55 = o_shift(a55, 48);
    { uint64_t t91 = a7; a7 = o_add(t91, a23); a23 = o_sub(t91, a23); }
    { uint64_t t92 = a39; a39 = o_add(t92, a55); a55 = o_sub(t92, a55); }
    { uint64_t t93 = a71; a71 = o_add(t93, a103); a103 = o_sub(t93, a103); }
    { uint64_t t94 = a87; a87 = o_add(t94, a119); a119 = o_sub(t94, a119); }
    a119 = o_shift(a119, 48);
    { uint64_t t95 = a71; a71 = o_add(t95, a87); a87 = o_sub(t95, a87); }
    { uint64_t t96 = a103; a103 = o_add(t96, a119); a119 = o_sub(t96, a119); }
    { uint64_t t97 = a8; a8 = o_add(t97, a72); a72 = o_sub(t97, a72); }
    { uint64_t t98 = a24; a24 = o_add(t98, a88); a88 = o_sub(t98, a88); }
    { uint64_t t99 = a40; a40 = o_add(t99, a104); a104 = o_sub(t99, a104); }
    { uint64_t t100 = a56; a56 = o_add(t100, a120); a120 = o_sub(t100, a120); }
    a88 = o_shift(a88, 24);
    a104 = o_shift(a104, 48);
    a120 = o_shift(a120, 72);
    { uint64_t t101 = a8; a8 = o_add(t101, a40); a40 = o_sub(t101, a40); }
    { uint64_t t102 = a24; a24 = o_add(t102, a56); a56 = o_sub(t102, a56); }
    a56 = o_shift(a56, 48);
    { uint64_t t103 = a8; a8 = o_add(t103, a24); a24 = o_sub(t103, a24); }
    { uint64_t t104 = a40; a40 = o_add(t104, a56); a56 = o_sub(t104, a56); }
    { uint64_t t105 = a72; a72 = o_add(t105, a104); a104 = o_sub(t105, a104); }
    { uint64_t t106 = a88; a88 = o_add(t106, a120); a120 = o_sub(t106, a120); }
    a120 = o_shift(a120, 48);
    { uint64_t t107 = a72; a72 = o_add(t107, a88); a88 = o_sub(t107, a88); }
    { uint64_t t108 = a104; a104 = o_add(t108, a120); a120 = o_sub(t108, a120); }
    { uint64_t t109 = a9; a9 = o_add(t109, a73); a73 = o_sub(t109, a73); }
    { uint64_t t110 = a25; a25 = o_add(t110, a89); a89 = o_sub(t110, a89); }
    { uint64_t t111 = a41; a41 = o_add(t111, a105); a105 = o_sub(t111, a105); }
    { uint64_t t112 = a57; a57 = o_add(t112, a121); a121 = o_sub(t112, a121); }
    a89 = o_shift(a89, 24);
    a105 = o_shift(a105, 48);
    a121 = o_shift(a121, 72);
    { uint64_t t113 = a9; a9 = o_add(t113, a41); a41 = o_sub(t113, a41); }
    { uint64_t t114 = a25; a25 = o_add(t114, a57); a57 = o_sub(t114, a57); }
    a57 = o_shift(a57, 48);
    { uint64_t t115 = a9; a9 = o_add(t115, a25); a25 = o_sub(t115, a25); }
    { uint64_t t116 = a41; a41 = o_add(t116, a57); a57 = o_sub(t116, a57); }
    { uint64_t t117 = a73; a73 = o_add(t117, a105); a105 = o_sub(t117, a105); }
    { uint64_t t118 = a89; a89 = o_add(t118, a121); a121 = o_sub(t118, a121); }
    a121 = o_shift(a121, 48);
    { uint64_t t119 = a73; a73 = o_add(t119, a89); a89 = o_sub(t119, a89); }
    { uint64_t t120 = a105; a105 = o_add(t120, a121); a121 = o_sub(t120, a121); }
    { uint64_t t121 = a10; a10 = o_add(t121, a74); a74 = o_sub(t121, a74); }
    { uint64_t t122 = a26; a26 = o_add(t122, a90); a90 = o_sub(t122, a90); }
    { uint64_t t123 = a42; a42 = o_add(t123, a106); a106 = o_sub(t123, a106); }
    { uint64_t t124 = a58; a58 = o_add(t124, a122); a122 = o_sub(t124, a122); }
    a90 = o_shift(a90, 24);
    a106 = o_shift(a106, 48);
    a122 = o_shift(a122, 72);
    { uint64_t t125 = a10; a10 = o_add(t125, a42); a42 = o_sub(t125, a42); }
    { uint64_t t126 = a26; a26 = o_add(t126, a58); a58 = o_sub(t126, a58); }
    a58 = o_shift(a58, 48);
    { uint64_t t127 = a10; a10 = o_add(t127, a26); a26 = o_sub(t127, a26); }
    { uint64_t t128 = a42; a42 = o_add(t128, a58); a58 = o_sub(t128, a58); }
    { uint64_t t129 = a74; a74 = o_add(t129, a106); a106 = o_sub(t129, a106); }
    { uint64_t t130 = a90; a90 = o_add(t130, a122); a122 = o_sub(t130, a122); }
    a122 = o_shift(a122, 48);
    { uint64_t t131 = a74; a74 = o_add(t131, a90); a90 = o_sub(t131, a90); }
    { uint64_t t132 = a106; a106 = o_add(t132, a122); a122 = o_sub(t132, a122); }
    { uint64_t t133 = a11; a11 = o_add(t133, a75); a75 = o_sub(t133, a75); }
    { uint64_t t134 = a27; a27 = o_add(t134, a91); a91 = o_sub(t134, a91); }
    { uint64_t t135 = a43; a43 = o_add(t135, a107); a107 = o_sub(t135, a107); }
    { uint64_t t136 = a59; a59 = o_add(t136, a123); a123 = o_sub(t136, a123); }
    a91 = o_shift(a91, 24);
    a107 = o_shift(a107, 48);
    a123 = o_shift(a123, 72);
    { uint64_t t137 = a11; a11 = o_add(t137, a43); a43 = o_sub(t137, a43); }
    { uint64_t t138 = a27; a27 = o_add(t138, a59); a59 = o_sub(t138, a59); }
    a59 = o_shift(a59, 48);
    { uint64_t t139 = a11; a11 = o_add(t139, a27); a27 = o_sub(t139, a27); }
    { uint64_t t140 = a43; a43 = o_add(t140, a59); a59 = o_sub(t140, a59); }
    { uint64_t t141 = a75; a75 = o_add(t141, a107); a107 = o_sub(t141, a107); }
    { uint64_t t142 = a91; a91 = o_add(t142, a123); a123 = o_sub(t142, a123); }
    a123 = o_shift(a123, 48);
    { uint64_t t143 = a75; a75 = o_add(t143, a91); a91 = o_sub(t143, a91); }
    { uint64_t t144 = a107; a107 = o_add(t144, a123); a123 = o_sub(t144, a123); }
    { uint64_t t145 = a12; a12 = o_add(t145, a76); a76 = o_sub(t145, a76); }
    { uint64_t t146 = a28; a28 = o_add(t146, a92); a92 = o_sub(t146, a92); }
    { uint64_t t147 = a44; a44 = o_add(t147, a108); a108 = o_sub(t147, a108); }
    { uint64_t t148 = a60; a60 = o_add(t148, a124); a124 = o_sub(t148, a124); }
    a92 = o_shift(a92, 24);
    a108 = o_shift(a108, 48);
    a124 = o_shift(a124, 72);
    { uint64_t t149 = a12; a12 = o_add(t149, a44); a44 = o_sub(t149, a44); }
    { uint64_t t150 = a28; a28 = o_add(t150, a60); a60 = o_sub(t150, a60); }
    a60 = o_shift(a60, 48);
    { uint64_t t151 = a12; a12 = o_add(t151, a28); a28 = o_sub(t151, a28); }
    { uint64_t t152 = a44; a44 = o_add(t152, a60); a60 = o_sub(t152, a60); }
    { uint64_t t153 = a76; a76 = o_add(t153, a108); a108 = o_sub(t153, a108); }
    { uint64_t t154 = a92; a92 = o_add(t154, a124); a124 = o_sub(t154, a124); }
    a124 = o_shift(a124, 48);
    { uint64_t t155 = a76; a76 = o_add(t155, a92); a92 = o_sub(t155, a92); }
    { uint64_t t156 = a108; a108 = o_add(t156, a124); a124 = o_sub(t156, a124); }
    { uint64_t t157 = a13; a13 = o_add(t157, a77); a77 = o_sub(t157, a77); }
    { uint64_t t158 = a29; a29 = o_add(t158, a93); a93 = o_sub(t158, a93); }
    { uint64_t t159 = a45; a45 = o_add(t159, a109); a109 = o_sub(t159, a109); }
    { uint64_t t160 = a61; a61 = o_add(t160, a125); a125 = o_sub(t160, a125); }
    a93 = o_shift(a93, 24);
    a109 = o_shift(a109, 48);
    a125 = o_shift(a125, 72);
    { uint64_t t161 = a13; a13 = o_add(t161, a45); a45 = o_sub(t161, a45); }
    { uint64_t t162 = a29; a29 = o_add(t162, a61); a61 = o_sub(t162, a61); }
    a61 = o_shift(a61, 48);
    { uint64_t t163 = a13; a13 = o_add(t163, a29); a29 = o_sub(t163, a29); }
    { uint64_t t164 = a45; a45 = o_add(t164, a61); a61 = o_sub(t164, a61); }
    { uint64_t t165 = a77; a77 = o_add(t165, a109); a109 = o_sub(t165, a109); }
    { uint64_t t166 = a93; a93 = o_add(t166, a125); a125 = o_sub(t166, a125); }
    a125 = o_shift(a125, 48);
    { uint64_t t167 = a77; a77 = o_add(t167, a93); a93 = o_sub(t167, a93); }
    { uint64_t t168 = a109; a109 = o_add(t168, a125); a125 = o_sub(t168, a125); }
    { uint64_t t169 = a14; a14 = o_add(t169, a78); a78 = o_sub(t169, a78); }
    { uint64_t t170 = a30; a30 = o_add(t170, a94); a94 = o_sub(t170, a94); }
    { uint64_t t171 = a46; a46 = o_add(t171, a110); a110 = o_sub(t171, a110); }
    { uint64_t t172 = a62; a62 = o_add(t172, a126); a126 = o_sub(t172, a126); }
    a94 = o_shift(a94, 24);
    a110 = o_shift(a110, 48);
    a126 = o_shift(a126, 72);
    { uint64_t t173 = a14; a14 = o_add(t173, a46); a46 = o_sub(t173, a46); }
    { uint64_t t174 = a30; a30 = o_add(t174, a62); a62 = o_sub(t174, a62); }
    a62 = o_shift(a62, 48);
    { uint64_t t175 = a14; a14 = o_add(t175, a30); a30 = o_sub(t175, a30); }
    { uint64_t t176 = a46; a46 = o_add(t176, a62); a62 = o_sub(t176, a62); }
    { uint64_t t177 = a78; a78 = o_add(t177, a110); a110 = o_sub(t177, a110); }
    { uint64_t t178 = a94; a94 = o_add(t178, a126); a126 = o_sub(t178, a126); }
    a126 = o_shift(a126, 48);
    { uint64_t t179 = a78; a78 = o_add(t179, a94); a94 = o_sub(t179, a94); }
    { uint64_t t180 = a110; a110 = o_add(t180, a126); a126 = o_sub(t180, a126); }
    { uint64_t t181 = a15; a15 = o_add(t181, a79); a79 = o_sub(t181, a79); }
    { uint64_t t182 = a31; a31 = o_add(t182, a95); a95 = o_sub(t182, a95); }
    { uint64_t t183 = a47; a47 = o_add(t183, a111); a111 = o_sub(t183, a111); }
    { uint64_t t184 = a63; a63 = o_add(t184, a127); a127 = o_sub(t184, a127); }
    a95 = o_shift(a95, 24);
    a111 = o_shift(a111, 48);
    a127 = o_shift(a127, 72);
    { uint64_t t185 = a15; a15 = o_add(t185, a47); a47 = o_sub(t185, a47); }
    { uint64_t t186 = a31; a31 = o_add(t186, a63); a63 = o_sub(t186, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t187 = a15; a15 = o_add(t187, a31); a31 = o_sub(t187, a31); }
    { uint64_t t188 = a47; a47 = o_add(t188, a63); a63 = o_sub(t188, a63); }
    { uint64_t t189 = a79; a79 = o_add(t189, a111); a111 = o_sub(t189, a111); }
    { uint64_t t190 = a95; a95 = o_add(t190, a127); a127 = o_sub(t190, a127); }
    a127 = o_shift(a127, 48);
    { uint64_t t191 = a79; a79 = o_add(t191, a95); a95 = o_sub(t191, a95); }
    { uint64_t t192 = a111; a111 = o_add(t192, a127); a127 = o_sub(t192, a127); }
    a65 = o_add(o_shift(a65, 25), o_neg(o_shift(a65, 73)));
    a33 = o_shift(a33, 3);
    a97 = o_add(o_shift(a97, 28), o_neg(o_shift(a97, 76)));
    a17 = o_shift(a17, 6);
    a81 = o_add(o_shift(a81, 31), o_neg(o_shift(a81, 79)));
    a49 = o_shift(a49, 9);
    a113 = o_add(o_shift(a113, 34), o_neg(o_shift(a113, 82)));
    a66 = o_shift(a66, 3);
    a34 = o_shift(a34, 6);
    a98 = o_shift(a98, 9);
    a18 = o_shift(a18, 12);
    a82 = o_shift(a82, 15);
    a50 = o_shift(a50, 18);
    a114 = o_shift(a114, 21);
    a67 = o_add(o_shift(a67, 28), o_neg(o_shift(a67, 76)));
    a35 = o_shift(a35, 9);
    a99 = o_add(o_shift(a99, 37), o_neg(o_shift(a99, 85)));
    a19 = o_shift(a19, 18);
    a83 = o_add(o_shift(a83, 46), o_neg(o_shift(a83, 94)));
    a51 = o_shift(a51, 27);
    a115 = o_add(o_shift(a115, 55), o_shift(a115, 7));
    a68 = o_shift(a68, 6);
    a36 = o_shift(a36, 12);
    a100 = o_shift(a100, 18);
    a20 = o_shift(a20, 24);
    a84 = o_shift(a84, 30);
    a52 = o_shift(a52, 36);
    a116 = o_shift(a116, 42);
    a69 = o_add(o_shift(a69, 31), o_neg(o_shift(a69, 79)));
    a37 = o_shift(a37, 15);
    a101 = o_add(o_shift(a101, 46), o_neg(o_shift(a101, 94)));
    a21 = o_shift(a21, 30);
    a85 = o_add(o_shift(a85, 61), o_shift(a85, 13));
    a53 = o_shift(a53, 45);
    a117 = o_add(o_shift(a117, 76), o_shift(a117, 28));
    a70 = o_shift(a70, 9);
    a38 = o_shift(a38, 18);
    a102 = o_shift(a102, 27);
    a22 = o_shift(a22, 36);
    a86 = o_shift(a86, 45);
    a54 = o_shift(a54, 54);
    a118 = o_shift(a118, 63);
    a71 = o_add(o_shift(a71, 34), o_neg(o_shift(a71, 82)));
    a39 = o_shift(a39, 21);
    a103 = o_add(o_shift(a103, 55), o_shift(a103, 7));
    a23 = o_shift(a23, 42);
    a87 = o_add(o_shift(a87, 76), o_shift(a87, 28));
    a55 = o_shift(a55, 63);
    a119 = o_add(o_neg(o_shift(a119, 1)), o_shift(a119, 49));
    a72 = o_shift(a72, 12);
    a40 = o_shift(a40, 24);
    a104 = o_shift(a104, 36);
    a24 = o_shift(a24, 48);
    a88 = o_shift(a88, 60);
    a56 = o_shift(a56, 72);
    a120 = o_shift(a120, 84);
    a73 = o_add(o_shift(a73, 37), o_neg(o_shift(a73, 85)));
    a41 = o_shift(a41, 27);
    a105 = o_add(o_shift(a105, 64), o_shift(a105, 16));
    a25 = o_shift(a25, 54);
    a89 = o_add(o_shift(a89, 91), o_shift(a89, 43));
    a57 = o_shift(a57, 81);
    a121 = o_add(o_neg(o_shift(a121, 22)), o_shift(a121, 70));
    a74 = o_shift(a74, 15);
    a42 = o_shift(a42, 30);
    a106 = o_shift(a106, 45);
    a26 = o_shift(a26, 60);
    a90 = o_shift(a90, 75);
    a58 = o_shift(a58, 90);
    a122 = o_neg(o_shift(a122, 9));
    a75 = o_add(o_shift(a75, 40), o_neg(o_shift(a75, 88)));
    a43 = o_shift(a43, 33);
    a107 = o_add(o_shift(a107, 73), o_shift(a107, 25));
    a27 = o_shift(a27, 66);
    a91 = o_add(o_neg(o_shift(a91, 10)), o_shift(a91, 58));
    a59 = o_neg(o_shift(a59, 3));
    a123 = o_add(o_neg(o_shift(a123, 43)), o_shift(a123, 91));
    a76 = o_shift(a76, 18);
    a44 = o_shift(a44, 36);
    a108 = o_shift(a108, 54);
    a28 = o_shift(a28, 72);
    a92 = o_shift(a92, 90);
    a60 = o_neg(o_shift(a60, 12));
    a124 = o_neg(o_shift(a124, 30));
    a77 = o_add(o_shift(a77, 43), o_neg(o_shift(a77, 91)));
    a45 = o_shift(a45, 39);
    a109 = o_add(o_shift(a109, 82), o_shift(a109, 34));
    a29 = o_shift(a29, 78);
    a93 = o_add(o_neg(o_shift(a93, 25)), o_shift(a93, 73));
    a61 = o_neg(o_shift(a61, 21));
    a125 = o_add(o_neg(o_shift(a125, 64)), o_neg(o_shift(a125, 16)));
    a78 = o_shift(a78, 21);
    a46 = o_shift(a46, 42);
    a110 = o_shift(a110, 63);
    a30 = o_shift(a30, 84);
    a94 = o_neg(o_shift(a94, 9));
    a62 = o_neg(o_shift(a62, 30));
    a126 = o_neg(o_shift(a126, 51));
    a79 = o_add(o_shift(a79, 46), o_neg(o_shift(a79, 94)));
    a47 = o_shift(a47, 45);
    a111 = o_add(o_shift(a111, 91), o_shift(a111, 43));
    a31 = o_shift(a31, 90);
    a95 = o_add(o_neg(o_shift(a95, 40)), o_shift(a95, 88));
    a63 = o_neg(o_shift(a63, 39));
    a127 = o_add(o_neg(o_shift(a127, 85)), o_neg(o_shift(a127, 37)));
    { uint64_t t193 = a0; a0 = o_add(t193, a8); a8 = o_sub(t193, a8); }
    { uint64_t t194 = a4; a4 = o_add(t194, a12); a12 = o_sub(t194, a12); }
    a12 = o_shift(a12, 48);
    { uint64_t t195 = a0; a0 = o_add(t195, a4); a4 = o_sub(t195, a4); }
    { uint64_t t196 = a8; a8 = o_add(t196, a12); a12 = o_sub(t196, a12); }
    { uint64_t t197 = a1; a1 = o_add(t197, a9); a9 = o_sub(t197, a9); }
    { uint64_t t198 = a5; a5 = o_add(t198, a13); a13 = o_sub(t198, a13); }
    a13 = o_shift(a13, 48);
    { uint64_t t199 = a1; a1 = o_add(t199, a5); a5 = o_sub(t199, a5); }
    { uint64_t t200 = a9; a9 = o_add(t200, a13); a13 = o_sub(t200, a13); }
    { uint64_t t201 = a2; a2 = o_add(t201, a10); a10 = o_sub(t201, a10); }
    { uint64_t t202 = a6; a6 = o_add(t202, a14); a14 = o_sub(t202, a14); }
    a14 = o_shift(a14, 48);
    { uint64_t t203 = a2; a2 = o_add(t203, a6); a6 = o_sub(t203, a6); }
    { uint64_t t204 = a10; a10 = o_add(t204, a14); a14 = o_sub(t204, a14); }
    { uint64_t t205 = a3; a3 = o_add(t205, a11); a11 = o_sub(t205, a11); }
    { uint64_t t206 = a7; a7 = o_add(t206, a15); a15 = o_sub(t206, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t207 = a3; a3 = o_add(t207, a7); a7 = o_sub(t207, a7); }
    { uint64_t t208 = a11; a11 = o_add(t208, a15); a15 = o_sub(t208, a15); }
    a9 = o_shift(a9, 12);
    a5 = o_shift(a5, 24);
    a13 = o_shift(a13, 36);
    a10 = o_shift(a10, 24);
    a6 = o_shift(a6, 48);
    a14 = o_shift(a14, 72);
    a11 = o_shift(a11, 36);
    a7 = o_shift(a7, 72);
    a15 = o_neg(o_shift(a15, 12));
    { uint64_t t209 = a0; a0 = o_add(t209, a2); a2 = o_sub(t209, a2); }
    { uint64_t t210 = a1; a1 = o_add(t210, a3); a3 = o_sub(t210, a3); }
    a3 = o_shift(a3, 48);
    { uint64_t t211 = a0; a0 = o_add(t211, a1); a1 = o_sub(t211, a1); }
    { uint64_t t212 = a2; a2 = o_add(t212, a3); a3 = o_sub(t212, a3); }
    { uint64_t t213 = a8; a8 = o_add(t213, a10); a10 = o_sub(t213, a10); }
    { uint64_t t214 = a9; a9 = o_add(t214, a11); a11 = o_sub(t214, a11); }
    a11 = o_shift(a11, 48);
    { uint64_t t215 = a8; a8 = o_add(t215, a9); a9 = o_sub(t215, a9); }
    { uint64_t t216 = a10; a10 = o_add(t216, a11); a11 = o_sub(t216, a11); }
    { uint64_t t217 = a4; a4 = o_add(t217, a6); a6 = o_sub(t217, a6); }
    { uint64_t t218 = a5; a5 = o_add(t218, a7); a7 = o_sub(t218, a7); }
    a7 = o_shift(a7, 48);
    { uint64_t t219 = a4; a4 = o_add(t219, a5); a5 = o_sub(t219, a5); }
    { uint64_t t220 = a6; a6 = o_add(t220, a7); a7 = o_sub(t220, a7); }
    { uint64_t t221 = a12; a12 = o_add(t221, a14); a14 = o_sub(t221, a14); }
    { uint64_t t222 = a13; a13 = o_add(t222, a15); a15 = o_sub(t222, a15); }
    a15 = o_shift(a15, 48);
    { uint64_t t223 = a12; a12 = o_add(t223, a13); a13 = o_sub(t223, a13); }
    { uint64_t t224 = a14; a14 = o_add(t224, a15); a15 = o_sub(t224, a15); }
    { uint64_t t225 = a64; a64 = o_add(t225, a72); a72 = o_sub(t225, a72); }
    { uint64_t t226 = a68; a68 = o_add(t226, a76); a76 = o_sub(t226, a76); }
    a76 = o_shift(a76, 48);
    { uint64_t t227 = a64; a64 = o_add(t227, a68); a68 = o_sub(t227, a68); }
    { uint64_t t228 = a72; a72 = o_add(t228, a76); a76 = o_sub(t228, a76); }
    { uint64_t t229 = a65; a65 = o_add(t229, a73); a73 = o_sub(t229, a73); }
    { uint64_t t230 = a69; a69 = o_add(t230, a77); a77 = o_sub(t230, a77); }
    a77 = o_shift(a77, 48);
    { uint64_t t231 = a65; a65 = o_add(t231, a69); a69 = o_sub(t231, a69); }
    { uint64_t t232 = a73; a73 = o_add(t232, a77); a77 = o_sub(t232, a77); }
    { uint64_t t233 = a66; a66 = o_add(t233, a74); a74 = o_sub(t233, a74); }
    { uint64_t t234 = a70; a70 = o_add(t234, a78); a78 = o_sub(t234, a78); }
    a78 = o_shift(a78, 48);
    { uint64_t t235 = a66; a66 = o_add(t235, a70); a70 = o_sub(t235, a70); }
    { uint64_t t236 = a74; a74 = o_add(t236, a78); a78 = o_sub(t236, a78); }
    { uint64_t t237 = a67; a67 = o_add(t237, a75); a75 = o_sub(t237, a75); }
    { uint64_t t238 = a71; a71 = o_add(t238, a79); a79 = o_sub(t238, a79); }
    a79 = o_shift(a79, 48);
    { uint64_t t239 = a67; a67 = o_add(t239, a71); a71 = o_sub(t239, a71); }
    { uint64_t t240 = a75; a75 = o_add(t240, a79); a79 = o_sub(t240, a79); }
    a73 = o_shift(a73, 12);
    a69 = o_shift(a69, 24);
    a77 = o_shift(a77, 36);
    a74 = o_shift(a74, 24);
    a70 = o_shift(a70, 48);
    a78 = o_shift(a78, 72);
    a75 = o_shift(a75, 36);
    a71 = o_shift(a71, 72);
    a79 = o_neg(o_shift(a79, 12));
    { uint64_t t241 = a64; a64 = o_add(t241, a66); a66 = o_sub(t241, a66); }
    { uint64_t t242 = a65; a65 = o_add(t242, a67); a67 = o_sub(t242, a67); }
    a67 = o_shift(a67, 48);
    { uint64_t t243 = a64; a64 = o_add(t243, a65); a65 = o_sub(t243, a65); }
    { uint64_t t244 = a66; a66 = o_add(t244, a67); a67 = o_sub(t244, a67); }
    { uint64_t t245 = a72; a72 = o_add(t245, a74); a74 = o_sub(t245, a74); }
    { uint64_t t246 = a73; a73 = o_add(t246, a75); a75 = o_sub(t246, a75); }
    a75 = o_shift(a75, 48);
    { uint64_t t247 = a72; a72 = o_add(t247, a73); a73 = o_sub(t247, a73); }
    { uint64_t t248 = a74; a74 = o_add(t248, a75); a75 = o_sub(t248, a75); }
    { uint64_t t249 = a68; a68 = o_add(t249, a70); a70 = o_sub(t249, a70); }
    { uint64_t t250 = a69; a69 = o_add(t250, a71); a71 = o_sub(t250, a71); }
    a71 = o_shift(a71, 48);
    { uint64_t t251 = a68; a68 = o_add(t251, a69); a69 = o_sub(t251, a69); }
    { uint64_t t252 = a70; a70 = o_add(t252, a71); a71 = o_sub(t252, a71); }
    { uint64_t t253 = a76; a76 = o_add(t253, a78); a78 = o_sub(t253, a78); }
    { uint64_t t254 = a77; a77 = o_add(t254, a79); a79 = o_sub(t254, a79); }
    a79 = o_shift(a79, 48);
    { uint64_t t255 = a76; a76 = o_add(t255, a77); a77 = o_sub(t255, a77); }
    { uint64_t t256 = a78; a78 = o_add(t256, a79); a79 = o_sub(t256, a79); }
    { uint64_t t257 = a32; a32 = o_add(t257, a40); a40 = o_sub(t257, a40); }
    { uint64_t t258 = a36; a36 = o_add(t258, a44); a44 = o_sub(t258, a44); }
    a44 = o_shift(a44, 48);
    { uint64_t t259 = a32; a32 = o_add(t259, a36); a36 = o_sub(t259, a36); }
    { uint64_t t260 = a40; a40 = o_add(t260, a44); a44 = o_sub(t260, a44); }
    { uint64_t t261 = a33; a33 = o_add(t261, a41); a41 = o_sub(t261, a41); }
    { uint64_t t262 = a37; a37 = o_add(t262, a45); a45 = o_sub(t262, a45); }
    a45 = o_shift(a45, 48);
    { uint64_t t263 = a33; a33 = o_add(t263, a37); a37 = o_sub(t263, a37); }
    { uint64_t t264 = a41; a41 = o_add(t264, a45); a45 = o_sub(t264, a45); }
    { uint64_t t265 = a34; a34 = o_add(t265, a42); a42 = o_sub(t265, a42); }
    { uint64_t t266 = a38; a38 = o_add(t266, a46); a46 = o_sub(t266, a46); }
    a46 = o_shift(a46, 48);
    { uint64_t t267 = a34; a34 = o_add(t267, a38); a38 = o_sub(t267, a38); }
    { uint64_t t268 = a42; a42 = o_add(t268, a46); a46 = o_sub(t268, a46); }
    { uint64_t t269 = a35; a35 = o_add(t269, a43); a43 = o_sub(t269, a43); }
    { uint64_t t270 = a39; a39 = o_add(t270, a47); a47 = o_sub(t270, a47); }
    a47 = o_shift(a47, 48);
    { uint64_t t271 = a35; a35 = o_add(t271, a39); a39 = o_sub(t271, a39); }
    { uint64_t t272 = a43; a43 = o_add(t272, a47); a47 = o_sub(t272, a47); }
    a41 = o_shift(a41, 12);
    a37 = o_shift(a37, 24);
    a45 = o_shift(a45, 36);
    a42 = o_shift(a42, 24);
    a38 = o_shift(a38, 48);
    a46 = o_shift(a46, 72);
    a43 = o_shift(a43, 36);
    a39 = o_shift(a39, 72);
    a47 = o_neg(o_shift(a47, 12));
    { uint64_t t273 = a32; a32 = o_add(t273, a34); a34 = o_sub(t273, a34); }
    { uint64_t t274 = a33; a33 = o_add(t274, a35); a35 = o_sub(t274, a35); }
    a35 = o_shift(a35, 48);
    { uint64_t t275 = a32; a32 = o_add(t275, a33); a33 = o_sub(t275, a33); }
    { uint64_t t276 = a34; a34 = o_add(t276, a35); a35 = o_sub(t276, a35); }
    { uint64_t t277 = a40; a40 = o_add(t277, a42); a42 = o_sub(t277, a42); }
    { uint64_t t278 = a41; a41 = o_add(t278, a43); a43 = o_sub(t278, a43); }
    a43 = o_shift(a43, 48);
    { uint64_t t279 = a40; a40 = o_add(t279, a41); a41 = o_sub(t279, a41); }
    { uint64_t t280 = a42; a42 = o_add(t280, a43); a43 = o_sub(t280, a43); }
    { uint64_t t281 = a36; a36 = o_add(t281, a38); a38 = o_sub(t281, a38); }
    { uint64_t t282 = a37; a37 = o_add(t282, a39); a39 = o_sub(t282, a39); }
    a39 = o_shift(a39, 48);
    { uint64_t t283 = a36; a36 = o_add(t283, a37); a37 = o_sub(t283, a37); }
    { uint64_t t284 = a38; a38 = o_add(t284, a39); a39 = o_sub(t284, a39); }
    { uint64_t t285 = a44; a44 = o_add(t285, a46); a46 = o_sub(t285, a46); }
    { uint64_t t286 = a45; a45 = o_add(t286, a47); a47 = o_sub(t286, a47); }
    a47 = o_shift(a47, 48);
    { uint64_t t287 = a44; a44 = o_add(t287, a45); a45 = o_sub(t287, a45); }
    { uint64_t t288 = a46; a46 = o_add(t288, a47); a47 = o_sub(t288, a47); }
    { uint64_t t289 = a96; a96 = o_add(t289, a104); a104 = o_sub(t289, a104); }
    { uint64_t t290 = a100; a100 = o_add(t290, a108); a108 = o_sub(t290, a108); }
    a108 = o_shift(a108, 48);
    { uint64_t t291 = a96; a96 = o_add(t291, a100); a100 = o_sub(t291, a100); }
    { uint64_t t292 = a104; a104 = o_add(t292, a108); a108 = o_sub(t292, a108); }
    { uint64_t t293 = a97; a97 = o_add(t293, a105); a105 = o_sub(t293, a105); }
    { uint64_t t294 = a101; a101 = o_add(t294, a109); a109 = o_sub(t294, a109); }
    a109 = o_shift(a109, 48);
    { uint64_t t295 = a97; a97 = o_add(t295, a101); a101 = o_sub(t295, a101); }
    { uint64_t t296 = a105; a105 = o_add(t296, a109); a109 = o_sub(t296, a109); }
    { uint64_t t297 = a98; a98 = o_add(t297, a106); a106 = o_sub(t297, a106); }
    { uint64_t t298 = a102; a102 = o_add(t298, a110); a110 = o_sub(t298, a110); }
    a110 = o_shift(a110, 48);
    { uint64_t t299 = a98; a98 = o_add(t299, a102); a102 = o_sub(t299, a102); }
    { uint64_t t300 = a106; a106 = o_add(t300, a110); a110 = o_sub(t300, a110); }
    { uint64_t t301 = a99; a99 = o_add(t301, a107); a107 = o_sub(t301, a107); }
    { uint64_t t302 = a103; a103 = o_add(t302, a111); a111 = o_sub(t302, a111); }
    a111 = o_shift(a111, 48);
    { uint64_t t303 = a99; a99 = o_add(t303, a103); a103 = o_sub(t303, a103); }
    { uint64_t t304 = a107; a107 = o_add(t304, a111); a111 = o_sub(t304, a111); }
    a105 = o_shift(a105, 12);
    a101 = o_shift(a101, 24);
    a109 = o_shift(a109, 36);
    a106 = o_shift(a106, 24);
    a102 = o_shift(a102, 48);
    a110 = o_shift(a110, 72);
    a107 = o_shift(a107, 36);
    a103 = o_shift(a103, 72);
    a111 = o_neg(o_shift(a111, 12));
    { uint64_t t305 = a96; a96 = o_add(t305, a98); a98 = o_sub(t305, a98); }
    { uint64_t t306 = a97; a97 = o_add(t306, a99); a99 = o_sub(t306, a99); }
    a99 = o_shift(a99, 48);
    { uint64_t t307 = a96; a96 = o_add(t307, a97); a97 = o_sub(t307, a97); }
    { uint64_t t308 = a98; a98 = o_add(t308, a99); a99 = o_sub(t308, a99); }
    { uint64_t t309 = a104; a104 = o_add(t309, a106); a106 = o_sub(t309, a106); }
    { uint64_t t310 = a105; a105 = o_add(t310, a107); a107 = o_sub(t310, a107); }
    a107 = o_shift(a107, 48);
    { uint64_t t311 = a104; a104 = o_add(t311, a105); a105 = o_sub(t311, a105); }
    { uint64_t t312 = a106; a106 = o_add(t312, a107); a107 = o_sub(t312, a107); }
    { uint64_t t313 = a100; a100 = o_add(t313, a102); a102 = o_sub(t313, a102); }
    { uint64_t t314 = a101; a101 = o_add(t314, a103); a103 = o_sub(t314, a103); }
    a103 = o_shift(a103, 48);
    { uint64_t t315 = a100; a100 = o_add(t315, a101); a101 = o_sub(t315, a101); }
    { uint64_t t316 = a102; a102 = o_add(t316, a103); a103 = o_sub(t316, a103); }
    { uint64_t t317 = a108; a108 = o_add(t317, a110); a110 = o_sub(t317, a110); }
    { uint64_t t318 = a109; a109 = o_add(t318, a111); a111 = o_sub(t318, a111); }
    a111 = o_shift(a111, 48);
    { uint64_t t319 = a108; a108 = o_add(t319, a109); a109 = o_sub(t319, a109); }
    { uint64_t t320 = a110; a110 = o_add(t320, a111); a111 = o_sub(t320, a111); }
    { uint64_t t321 = a16; a16 = o_add(t321, a24); a24 = o_sub(t321, a24); }
    { uint64_t t322 = a20; a20 = o_add(t322, a28); a28 = o_sub(t322, a28); }
    a28 = o_shift(a28, 48);
    { uint64_t t323 = a16; a16 = o_add(t323, a20); a20 = o_sub(t323, a20); }
    { uint64_t t324 = a24; a24 = o_add(t324, a28); a28 = o_sub(t324, a28); }
    { uint64_t t325 = a17; a17 = o_add(t325, a25); a25 = o_sub(t325, a25); }
    { uint64_t t326 = a21; a21 = o_add(t326, a29); a29 = o_sub(t326, a29); }
    a29 = o_shift(a29, 48);
    { uint64_t t327 = a17; a17 = o_add(t327, a21); a21 = o_sub(t327, a21); }
    { uint64_t t328 = a25; a25 = o_add(t328, a29); a29 = o_sub(t328, a29); }
    { uint64_t t329 = a18; a18 = o_add(t329, a26); a26 = o_sub(t329, a26); }
    { uint64_t t330 = a22; a22 = o_add(t330, a30); a30 = o_sub(t330, a30); }
    a30 = o_shift(a30, 48);
    { uint64_t t331 = a18; a18 = o_add(t331, a22); a22 = o_sub(t331, a22); }
    { uint64_t t332 = a26; a26 = o_add(t332, a30); a30 = o_sub(t332, a30); }
    { uint64_t t333 = a19; a19 = o_add(t333, a27); a27 = o_sub(t333, a27); }
    { uint64_t t334 = a23; a23 = o_add(t334, a31); a31 = o_sub(t334, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t335 = a19; a19 = o_add(t335, a23); a23 = o_sub(t335, a23); }
    { uint64_t t336 = a27; a27 = o_add(t336, a31); a31 = o_sub(t336, a31); }
    a25 = o_shift(a25, 12);
    a21 = o_shift(a21, 24);
    a29 = o_shift(a29, 36);
    a26 = o_shift(a26, 24);
    a22 = o_shift(a22, 48);
    a30 = o_shift(a30, 72);
    a27 = o_shift(a27, 36);
    a23 = o_shift(a23, 72);
    a31 = o_neg(o_shift(a31, 12));
    { uint64_t t337 = a16; a16 = o_add(t337, a18); a18 = o_sub(t337, a18); }
    { uint64_t t338 = a17; a17 = o_add(t338, a19); a19 = o_sub(t338, a19); }
    a19 = o_shift(a19, 48);
    { uint64_t t339 = a16; a16 = o_add(t339, a17); a17 = o_sub(t339, a17); }
    { uint64_t t340 = a18; a18 = o_add(t340, a19); a19 = o_sub(t340, a19); }
    { uint64_t t341 = a24; a24 = o_add(t341, a26); a26 = o_sub(t341, a26); }
    { uint64_t t342 = a25; a25 = o_add(t342, a27); a27 = o_sub(t342, a27); }
    a27 = o_shift(a27, 48);
    { uint64_t t343 = a24; a24 = o_add(t343, a25); a25 = o_sub(t343, a25); }
    { uint64_t t344 = a26; a26 = o_add(t344, a27); a27 = o_sub(t344, a27); }
    { uint64_t t345 = a20; a20 = o_add(t345, a22); a22 = o_sub(t345, a22); }
    { uint64_t t346 = a21; a21 = o_add(t346, a23); a23 = o_sub(t346, a23); }
    a23 = o_shift(a23, 48);
    { uint64_t t347 = a20; a20 = o_add(t347, a21); a21 = o_sub(t347, a21); }
    { uint64_t t348 = a22; a22 = o_add(t348, a23); a23 = o_sub(t348, a23); }
    { uint64_t t349 = a28; a28 = o_add(t349, a30); a30 = o_sub(t349, a30); }
    { uint64_t t350 = a29; a29 = o_add(t350, a31); a31 = o_sub(t350, a31); }
    a31 = o_shift(a31, 48);
    { uint64_t t351 = a28; a28 = o_add(t351, a29); a29 = o_sub(t351, a29); }
    { uint64_t t352 = a30; a30 = o_add(t352, a31); a31 = o_sub(t352, a31); }
    { uint64_t t353 = a80; a80 = o_add(t353, a88); a88 = o_sub(t353, a88); }
    { uint64_t t354 = a84; a84 = o_add(t354, a92); a92 = o_sub(t354, a92); }
    a92 = o_shift(a92, 48);
    { uint64_t t355 = a80; a80 = o_add(t355, a84); a84 = o_sub(t355, a84); }
    { uint64_t t356 = a88; a88 = o_add(t356, a92); a92 = o_sub(t356, a92); }
    { uint64_t t357 = a81; a81 = o_add(t357, a89); a89 = o_sub(t357, a89); }
    { uint64_t t358 = a85; a85 = o_add(t358, a93); a93 = o_sub(t358, a93); }
    a93 = o_shift(a93, 48);
    { uint64_t t359 = a81; a81 = o_add(t359, a85); a85 = o_sub(t359, a85); }
    { uint64_t t360 = a89; a89 = o_add(t360, a93); a93 = o_sub(t360, a93); }
    { uint64_t t361 = a82; a82 = o_add(t361, a90); a90 = o_sub(t361, a90); }
    { uint64_t t362 = a86; a86 = o_add(t362, a94); a94 = o_sub(t362, a94); }
    a94 = o_shift(a94, 48);
    { uint64_t t363 = a82; a82 = o_add(t363, a86); a86 = o_sub(t363, a86); }
    { uint64_t t364 = a90; a90 = o_add(t364, a94); a94 = o_sub(t364, a94); }
    { uint64_t t365 = a83; a83 = o_add(t365, a91); a91 = o_sub(t365, a91); }
    { uint64_t t366 = a87; a87 = o_add(t366, a95); a95 = o_sub(t366, a95); }
    a95 = o_shift(a95, 48);
    { uint64_t t367 = a83; a83 = o_add(t367, a87); a87 = o_sub(t367, a87); }
    { uint64_t t368 = a91; a91 = o_add(t368, a95); a95 = o_sub(t368, a95); }
    a89 = o_shift(a89, 12);
    a85 = o_shift(a85, 24);
    a93 = o_shift(a93, 36);
    a90 = o_shift(a90, 24);
    a86 = o_shift(a86, 48);
    a94 = o_shift(a94, 72);
    a91 = o_shift(a91, 36);
    a87 = o_shift(a87, 72);
    a95 = o_neg(o_shift(a95, 12));
    { uint64_t t369 = a80; a80 = o_add(t369, a82); a82 = o_sub(t369, a82); }
    { uint64_t t370 = a81; a81 = o_add(t370, a83); a83 = o_sub(t370, a83); }
    a83 = o_shift(a83, 48);
    { uint64_t t371 = a80; a80 = o_add(t371, a81); a81 = o_sub(t371, a81); }
    { uint64_t t372 = a82; a82 = o_add(t372, a83); a83 = o_sub(t372, a83); }
    { uint64_t t373 = a88; a88 = o_add(t373, a90); a90 = o_sub(t373, a90); }
    { uint64_t t374 = a89; a89 = o_add(t374, a91); a91 = o_sub(t374, a91); }
    a91 = o_shift(a91, 48);
    { uint64_t t375 = a88; a88 = o_add(t375, a89); a89 = o_sub(t375, a89); }
    { uint64_t t376 = a90; a90 = o_add(t376, a91); a91 = o_sub(t376, a91); }
    { uint64_t t377 = a84; a84 = o_add(t377, a86); a86 = o_sub(t377, a86); }
    { uint64_t t378 = a85; a85 = o_add(t378, a87); a87 = o_sub(t378, a87); }
    a87 = o_shift(a87, 48);
    { uint64_t t379 = a84; a84 = o_add(t379, a85); a85 = o_sub(t379, a85); }
    { uint64_t t380 = a86; a86 = o_add(t380, a87); a87 = o_sub(t380, a87); }
    { uint64_t t381 = a92; a92 = o_add(t381, a94); a94 = o_sub(t381, a94); }
    { uint64_t t382 = a93; a93 = o_add(t382, a95); a95 = o_sub(t382, a95); }
    a95 = o_shift(a95, 48);
    { uint64_t t383 = a92; a92 = o_add(t383, a93); a93 = o_sub(t383, a93); }
    { uint64_t t384 = a94; a94 = o_add(t384, a95); a95 = o_sub(t384, a95); }
    { uint64_t t385 = a48; a48 = o_add(t385, a56); a56 = o_sub(t385, a56); }
    { uint64_t t386 = a52; a52 = o_add(t386, a60); a60 = o_sub(t386, a60); }
    a60 = o_shift(a60, 48);
    { uint64_t t387 = a48; a48 = o_add(t387, a52); a52 = o_sub(t387, a52); }
    { uint64_t t388 = a56; a56 = o_add(t388, a60); a60 = o_sub(t388, a60); }
    { uint64_t t389 = a49; a49 = o_add(t389, a57); a57 = o_sub(t389, a57); }
    { uint64_t t390 = a53; a53 = o_add(t390, a61); a61 = o_sub(t390, a61); }
    a61 = o_shift(a61, 48);
    { uint64_t t391 = a49; a49 = o_add(t391, a53); a53 = o_sub(t391, a53); }
    { uint64_t t392 = a57; a57 = o_add(t392, a61); a61 = o_sub(t392, a61); }
    { uint64_t t393 = a50; a50 = o_add(t393, a58); a58 = o_sub(t393, a58); }
    { uint64_t t394 = a54; a54 = o_add(t394, a62); a62 = o_sub(t394, a62); }
    a62 = o_shift(a62, 48);
    { uint64_t t395 = a50; a50 = o_add(t395, a54); a54 = o_sub(t395, a54); }
    { uint64_t t396 = a58; a58 = o_add(t396, a62); a62 = o_sub(t396, a62); }
    { uint64_t t397 = a51; a51 = o_add(t397, a59); a59 = o_sub(t397, a59); }
    { uint64_t t398 = a55; a55 = o_add(t398, a63); a63 = o_sub(t398, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t399 = a51; a51 = o_add(t399, a55); a55 = o_sub(t399, a55); }
    { uint64_t t400 = a59; a59 = o_add(t400, a63); a63 = o_sub(t400, a63); }
    a57 = o_shift(a57, 12);
    a53 = o_shift(a53, 24);
    a61 = o_shift(a61, 36);
    a58 = o_shift(a58, 24);
    a54 = o_shift(a54, 48);
    a62 = o_shift(a62, 72);
    a59 = o_shift(a59, 36);
    a55 = o_shift(a55, 72);
    a63 = o_neg(o_shift(a63, 12));
    { uint64_t t401 = a48; a48 = o_add(t401, a50); a50 = o_sub(t401, a50); }
    { uint64_t t402 = a49; a49 = o_add(t402, a51); a51 = o_sub(t402, a51); }
    a51 = o_shift(a51, 48);
    { uint64_t t403 = a48; a48 = o_add(t403, a49); a49 = o_sub(t403, a49); }
    { uint64_t t404 = a50; a50 = o_add(t404, a51); a51 = o_sub(t404, a51); }
    { uint64_t t405 = a56; a56 = o_add(t405, a58); a58 = o_sub(t405, a58); }
    { uint64_t t406 = a57; a57 = o_add(t406, a59); a59 = o_sub(t406, a59); }
    a59 = o_shift(a59, 48);
    { uint64_t t407 = a56; a56 = o_add(t407, a57); a57 = o_sub(t407, a57); }
    { uint64_t t408 = a58; a58 = o_add(t408, a59); a59 = o_sub(t408, a59); }
    { uint64_t t409 = a52; a52 = o_add(t409, a54); a54 = o_sub(t409, a54); }
    { uint64_t t410 = a53; a53 = o_add(t410, a55); a55 = o_sub(t410, a55); }
    a55 = o_shift(a55, 48);
    { uint64_t t411 = a52; a52 = o_add(t411, a53); a53 = o_sub(t411, a53); }
    { uint64_t t412 = a54; a54 = o_add(t412, a55); a55 = o_sub(t412, a55); }
    { uint64_t t413 = a60; a60 = o_add(t413, a62); a62 = o_sub(t413, a62); }
    { uint64_t t414 = a61; a61 = o_add(t414, a63); a63 = o_sub(t414, a63); }
    a63 = o_shift(a63, 48);
    { uint64_t t415 = a60; a60 = o_add(t415, a61); a61 = o_sub(t415, a61); }
    { uint64_t t416 = a62; a62 = o_add(t416, a63); a63 = o_sub(t416, a63); }
    { uint64_t t417 = a112; a112 = o_add(t417, a120); a120 = o_sub(t417, a120); }
    { uint64_t t418 = a116; a116 = o_add(t418, a124); a124 = o_sub(t418, a124); }
    a124 = o_shift(a124, 48);
    { uint64_t t419 = a112; a112 = o_add(t419, a116); a116 = o_sub(t419, a116); }
    { uint64_t t420 = a120; a120 = o_add(t420, a124); a124 = o_sub(t420, a124); }
    { uint64_t t421 = a113; a113 = o_add(t421, a121); a121 = o_sub(t421, a121); }
    { uint64_t t422 = a117; a117 = o_add(t422, a125); a125 = o_sub(t422, a125); }
    a125 = o_shift(a125, 48);
    { uint64_t t423 = a113; a113 = o_add(t423, a117); a117 = o_sub(t423, a117); }
    { uint64_t t424 = a121; a121 = o_add(t424, a125); a125 = o_sub(t424, a125); }
    { uint64_t t425 = a114; a114 = o_add(t425, a122); a122 = o_sub(t425, a122); }
    { uint64_t t426 = a118; a118 = o_add(t426, a126); a126 = o_sub(t426, a126); }
    a126 = o_shift(a126, 48);
    { uint64_t t427 = a114; a114 = o_add(t427, a118); a118 = o_sub(t427, a118); }
    { uint64_t t428 = a122; a122 = o_add(t428, a126); a126 = o_sub(t428, a126); }
    { uint64_t t429 = a115; a115 = o_add(t429, a123); a123 = o_sub(t429, a123); }
    { uint64_t t430 = a119; a119 = o_add(t430, a127); a127 = o_sub(t430, a127); }
    a127 = o_shift(a127, 48);
    { uint64_t t431 = a115; a115 = o_add(t431, a119); a119 = o_sub(t431, a119); }
    { uint64_t t432 = a123; a123 = o_add(t432, a127); a127 = o_sub(t432, a127); }
    a121 = o_shift(a121, 12);
    a117 = o_shift(a117, 24);
    a125 = o_shift(a125, 36);
    a122 = o_shift(a122, 24);
    a118 = o_shift(a118, 48);
    a126 = o_shift(a126, 72);
    a123 = o_shift(a123, 36);
    a119 = o_shift(a119, 72);
    a127 = o_neg(o_shift(a127, 12));
    { uint64_t t433 = a112; a112 = o_add(t433, a114); a114 = o_sub(t433, a114); }
    { uint64_t t434 = a113; a113 = o_add(t434, a115); a115 = o_sub(t434, a115); }
    a115 = o_shift(a115, 48);
    { uint64_t t435 = a112; a112 = o_add(t435, a113); a113 = o_sub(t435, a113); }
    { uint64_t t436 = a114; a114 = o_add(t436, a115); a115 = o_sub(t436, a115); }
    { uint64_t t437 = a120; a120 = o_add(t437, a122); a122 = o_sub(t437, a122); }
    { uint64_t t438 = a121; a121 = o_add(t438, a123); a123 = o_sub(t438, a123); }
    a123 = o_shift(a123, 48);
    { uint64_t t439 = a120; a120 = o_add(t439, a121); a121 = o_sub(t439, a121); }
    { uint64_t t440 = a122; a122 = o_add(t440, a123); a123 = o_sub(t440, a123); }
    { uint64_t t441 = a116; a116 = o_add(t441, a118); a118 = o_sub(t441, a118); }
    { uint64_t t442 = a117; a117 = o_add(t442, a119); a119 = o_sub(t442, a119); }
    a119 = o_shift(a119, 48);
    { uint64_t t443 = a116; a116 = o_add(t443, a117); a117 = o_sub(t443, a117); }
    { uint64_t t444 = a118; a118 = o_add(t444, a119); a119 = o_sub(t444, a119); }
    { uint64_t t445 = a124; a124 = o_add(t445, a126); a126 = o_sub(t445, a126); }
    { uint64_t t446 = a125; a125 = o_add(t446, a127); a127 = o_sub(t446, a127); }
    a127 = o_shift(a127, 48);
    { uint64_t t447 = a124; a124 = o_add(t447, a125); a125 = o_sub(t447, a125); }
    { uint64_t t448 = a126; a126 = o_add(t448, a127); a127 = o_sub(t448, a127); }
    v[0] = a0;
    v[1] = a64;
    v[2] = a32;
    v[3] = a96;
    v[4] = a16;
    v[5] = a80;
    v[6] = a48;
    v[7] = a112;
    v[8] = a8;
    v[9] = a72;
    v[10] = a40;
    v[11] = a104;
    v[12] = a24;
    v[13] = a88;
    v[14] = a56;
    v[15] = a120;
    v[16] = a4;
    v[17] = a68;
    v[18] = a36;
    v[19] = a100;
    v[20] = a20;
    v[21] = a84;
    v[22] = a52;
    v[23] = a116;
    v[24] = a12;
    v[25] = a76;
    v[26] = a44;
    v[27] = a108;
    v[28] = a28;
    v[29] = a92;
    v[30] = a60;
    v[31] = a124;
    v[32] = a2;
    v[33] = a66;
    v[34] = a34;
    v[35] = a98;
    v[36] = a18;
    v[37] = a82;
    v[38] = a50;
    v[39] = a114;
    v[40] = a10;
    v[41] = a74;
    v[42] = a42;
    v[43] = a106;
    v[44] = a26;
    v[45] = a90;
    v[46] = a58;
    v[47] = a122;
    v[48] = a6;
    v[49] = a70;
    v[50] = a38;
    v[51] = a102;
    v[52] = a22;
    v[53] = a86;
    v[54] = a54;
    v[55] = a118;
    v[56] = a14;
    v[57] = a78;
    v[58] = a46;
    v[59] = a110;
    v[60] = a30;
    v[61] = a94;
    v[62] = a62;
    v[63] = a126;
    v[64] = a1;
    v[65] = a65;
    v[66] = a33;
    v[67] = a97;
    v[68] = a17;
    v[69] = a81;
    v[70] = a49;
    v[71] = a113;
    v[72] = a9;
    v[73] = a73;
    v[74] = a41;
    v[75] = a105;
    v[76] = a25;
    v[77] = a89;
    v[78] = a57;
    v[79] = a121;
    v[80] = a5;
    v[81] = a69;
    v[82] = a37;
    v[83] = a101;
    v[84] = a21;
    v[85] = a85;
    v[86] = a53;
    v[87] = a117;
    v[88] = a13;
    v[89] = a77;
    v[90] = a45;
    v[91] = a109;
    v[92] = a29;
    v[93] = a93;
    v[94] = a61;
    v[95] = a125;
    v[96] = a3;
    v[97] = a67;
    v[98] = a35;
    v[99] = a99;
    v[100] = a19;
    v[101] = a83;
    v[102] = a51;
    v[103] = a115;
    v[104] = a11;
    v[105] = a75;
    v[106] = a43;
    v[107] = a107;
    v[108] = a27;
    v[109] = a91;
    v[110] = a59;
    v[111] = a123;
    v[112] = a7;
    v[113] = a71;
    v[114] = a39;
    v[115] = a103;
    v[116] = a23;
    v[117] = a87;
    v[118] = a55;
    v[119] = a119;
    v[120] = a15;
    v[121] = a79;
    v[122] = a47;
    v[123] = a111;
    v[124] = a31;
    v[125] = a95;
    v[126] = a63;
    v[127] = a127;
}

o_codelet_fn o_small_codelet(uint64_t size) {
    switch (size) {
    case 2: return o_ntt_2;
    case 3: return o_ntt_3;
    case 4: return o_ntt_4;
    case 5: return o_ntt_5;
    case 6: return o_ntt_6;
    case 8: return o_ntt_8;
    case 10: return o_ntt_10;
    case 12: return o_ntt_12;
    case 15: return o_ntt_15;
    case 16: return o_ntt_16;
    case 17: return o_ntt_17;
    case 20: return o_ntt_20;
    case 24: return o_ntt_24;
    case 30: return o_ntt_30;
    case 32: return o_ntt_32;
    case 34: return o_ntt_34;
    case 40: return o_ntt_40;
    case 48: return o_ntt_48;
    case 51: return o_ntt_51;
    case 60: return o_ntt_60;
    case 64: return o_ntt_64;
    case 68: return o_ntt_68;
    case 80: return o_ntt_80;
    case 85: return o_ntt_85;
    case 96: return o_ntt_96;
    case 102: return o_ntt_102;
    case 120: return o_ntt_120;
    case 128: return o_ntt_128;
    default: return 0;
    }
}
