// Butcher tables of the Runge-Kutta methods the reference's input files select, by their
// ARKODE table numbers (the `etable` / `itable` options, src/euler3D.hpp:126-172, passed to
// ARKStepSetTableNum in src/euler3D_main.cpp:209-213, src/imex_chem_hydro_main.cpp:386 and
// src/multirate_chem_hydro_main.cpp:447; `order` picks ARKODE's default table of that order).
// Coefficients are the published ones, each rational written as the quotient of its two
// integers (evaluated once in double, as a compiled-in table would be):
//   0  Heun-Euler 2(1)                      (Heun; Euler embedding)
//   1  Bogacki-Shampine 3(2)                (P. Bogacki, L. F. Shampine, Appl. Math. Lett. 2
//                                             (1989) 321-325)
//   2  ARK3(2)4L[2]SA, explicit part         (C. A. Kennedy, M. H. Carpenter, Appl. Numer.
//   104 ARK3(2)4L[2]SA, implicit part          Math. 44 (2003) 139-181)
//   3  Zonneveld 4(3)                       (J. A. Zonneveld, Automatic numerical integration,
//                                             Math. Centre Tracts 8, Amsterdam 1964)
//   6  Cash-Karp 5(4)                       (J. R. Cash, A. H. Karp, ACM TOMS 16 (1990) 201-222)
//   8  Dormand-Prince 5(4)                  (J. R. Dormand, P. J. Prince, J. Comput. Appl.
//                                             Math. 6 (1980) 19-26)
//   13 ARK4(3)7L[2]SA, explicit part        (C. A. Kennedy, M. H. Carpenter, Appl. Numer.
//   112 ARK4(3)7L[2]SA, implicit part         Math. 136 (2019) 183-205)
//   102 TR-BDF2 as a 3-stage ESDIRK 2(3)     (M. E. Hosea, L. F. Shampine, Appl. Numer. Math.
//                                             20 (1996) 21-37)
// The pairs (2, 104) and (13, 112) share c and b, so either pair is an additive (IMEX) method.
#include <string.h>

#include "butcher.cuh"

namespace gbmv {
namespace {

#define Q(a, b) (double(a) / double(b))

constexpr double kRt2 = 1.4142135623730951;  // sqrt(2) rounded to double

ButcherTable make(int id, const char* name, int s, int q, int p) {
  ButcherTable t;
  memset(&t, 0, sizeof t);
  t.id = id;
  t.name = name;
  t.s = s;
  t.q = q;
  t.p = p;
  return t;
}

ButcherTable heun_euler() {
  ButcherTable t = make(0, "HEUN_EULER_2_1_2", 2, 2, 1);
  t.c[1] = 1.0;
  t.A[1][0] = 1.0;
  t.b[0] = 0.5; t.b[1] = 0.5;
  t.bhat[0] = 1.0;
  return t;
}

ButcherTable bogacki_shampine() {
  ButcherTable t = make(1, "BOGACKI_SHAMPINE_4_2_3", 4, 3, 2);
  t.c[1] = 0.5; t.c[2] = 0.75; t.c[3] = 1.0;
  t.A[1][0] = 0.5;
  t.A[2][1] = 0.75;
  t.A[3][0] = Q(2, 9); t.A[3][1] = Q(1, 3); t.A[3][2] = Q(4, 9);
  t.b[0] = Q(2, 9); t.b[1] = Q(1, 3); t.b[2] = Q(4, 9);
  t.bhat[0] = Q(7, 24); t.bhat[1] = 0.25; t.bhat[2] = Q(1, 3); t.bhat[3] = 0.125;
  return t;
}

// c and b shared by both parts of ARK3(2)4L[2]SA
void ark324_common(ButcherTable& t) {
  t.c[1] = Q(1767732205903LL, 2027836641118LL); t.c[2] = Q(3, 5); t.c[3] = 1.0;
  t.b[0] = Q(1471266399579LL, 7840856788654LL);
  t.b[1] = Q(-4482444167858LL, 7529755066697LL);
  t.b[2] = Q(11266239266428LL, 11593286722821LL);
  t.b[3] = Q(1767732205903LL, 4055673282236LL);
  t.bhat[0] = Q(2756255671327LL, 12835298489170LL);
  t.bhat[1] = Q(-10771552573575LL, 22201958757719LL);
  t.bhat[2] = Q(9247589265047LL, 10645013368117LL);
  t.bhat[3] = Q(2193209047091LL, 5459859503100LL);
}

ButcherTable ark324_erk() {
  ButcherTable t = make(2, "ARK324L2SA_ERK_4_2_3", 4, 3, 2);
  ark324_common(t);
  t.A[1][0] = Q(1767732205903LL, 2027836641118LL);
  t.A[2][0] = Q(5535828885825LL, 10492691773637LL);
  t.A[2][1] = Q(788022342437LL, 10882634858940LL);
  t.A[3][0] = Q(6485989280629LL, 16251701735622LL);
  t.A[3][1] = Q(-4246266847089LL, 9704473918619LL);
  t.A[3][2] = Q(10755448449292LL, 10357097424841LL);
  return t;
}

ButcherTable ark324_dirk() {
  ButcherTable t = make(104, "ARK324L2SA_DIRK_4_2_3", 4, 3, 2);
  ark324_common(t);
  const double g = Q(1767732205903LL, 4055673282236LL);
  t.A[1][0] = g; t.A[1][1] = g;
  t.A[2][0] = Q(2746238789719LL, 10658868560708LL);
  t.A[2][1] = Q(-640167445237LL, 6845629431997LL);
  t.A[2][2] = g;
  for (int j = 0; j < 4; ++j) t.A[3][j] = t.b[j];
  return t;
}

ButcherTable zonneveld() {
  ButcherTable t = make(3, "ZONNEVELD_5_3_4", 5, 4, 3);
  t.c[1] = 0.5; t.c[2] = 0.5; t.c[3] = 1.0; t.c[4] = 0.75;
  t.A[1][0] = 0.5;
  t.A[2][1] = 0.5;
  t.A[3][2] = 1.0;
  t.A[4][0] = Q(5, 32); t.A[4][1] = Q(7, 32); t.A[4][2] = Q(13, 32); t.A[4][3] = Q(-1, 32);
  t.b[0] = Q(1, 6); t.b[1] = Q(1, 3); t.b[2] = Q(1, 3); t.b[3] = Q(1, 6);
  t.bhat[0] = Q(-1, 2); t.bhat[1] = Q(7, 3); t.bhat[2] = Q(7, 3); t.bhat[3] = Q(13, 6);
  t.bhat[4] = Q(-16, 3);
  return t;
}

ButcherTable cash_karp() {
  ButcherTable t = make(6, "CASH_KARP_6_4_5", 6, 5, 4);
  t.c[1] = Q(1, 5); t.c[2] = Q(3, 10); t.c[3] = Q(3, 5); t.c[4] = 1.0; t.c[5] = Q(7, 8);
  t.A[1][0] = Q(1, 5);
  t.A[2][0] = Q(3, 40); t.A[2][1] = Q(9, 40);
  t.A[3][0] = Q(3, 10); t.A[3][1] = Q(-9, 10); t.A[3][2] = Q(6, 5);
  t.A[4][0] = Q(-11, 54); t.A[4][1] = Q(5, 2); t.A[4][2] = Q(-70, 27); t.A[4][3] = Q(35, 27);
  t.A[5][0] = Q(1631, 55296); t.A[5][1] = Q(175, 512); t.A[5][2] = Q(575, 13824);
  t.A[5][3] = Q(44275, 110592); t.A[5][4] = Q(253, 4096);
  t.b[0] = Q(37, 378); t.b[2] = Q(250, 621); t.b[3] = Q(125, 594); t.b[5] = Q(512, 1771);
  t.bhat[0] = Q(2825, 27648); t.bhat[2] = Q(18575, 48384); t.bhat[3] = Q(13525, 55296);
  t.bhat[4] = Q(277, 14336); t.bhat[5] = 0.25;
  return t;
}

ButcherTable dormand_prince() {
  ButcherTable t = make(8, "DORMAND_PRINCE_7_4_5", 7, 5, 4);
  t.c[1] = Q(1, 5); t.c[2] = Q(3, 10); t.c[3] = Q(4, 5); t.c[4] = Q(8, 9); t.c[5] = 1.0;
  t.c[6] = 1.0;
  t.A[1][0] = Q(1, 5);
  t.A[2][0] = Q(3, 40); t.A[2][1] = Q(9, 40);
  t.A[3][0] = Q(44, 45); t.A[3][1] = Q(-56, 15); t.A[3][2] = Q(32, 9);
  t.A[4][0] = Q(19372, 6561); t.A[4][1] = Q(-25360, 2187); t.A[4][2] = Q(64448, 6561);
  t.A[4][3] = Q(-212, 729);
  t.A[5][0] = Q(9017, 3168); t.A[5][1] = Q(-355, 33); t.A[5][2] = Q(46732, 5247);
  t.A[5][3] = Q(49, 176); t.A[5][4] = Q(-5103, 18656);
  t.A[6][0] = Q(35, 384); t.A[6][2] = Q(500, 1113); t.A[6][3] = Q(125, 192);
  t.A[6][4] = Q(-2187, 6784); t.A[6][5] = Q(11, 84);
  for (int j = 0; j < 7; ++j) t.b[j] = t.A[6][j];
  t.bhat[0] = Q(5179, 57600); t.bhat[2] = Q(7571, 16695); t.bhat[3] = Q(393, 640);
  t.bhat[4] = Q(-92097, 339200); t.bhat[5] = Q(187, 2100); t.bhat[6] = Q(1, 40);
  return t;
}

// c and b shared by both parts of ARK4(3)7L[2]SA
void ark437_common(ButcherTable& t) {
  t.c[1] = Q(247, 1000);
  t.c[2] = Q(4276536705230LL, 10142255878289LL);
  t.c[3] = Q(67, 200);
  t.c[4] = Q(3, 40);
  t.c[5] = Q(7, 10);
  t.c[6] = 1.0;
  t.b[2] = Q(9164257142617LL, 17756377923965LL);
  t.b[3] = Q(-10812980402763LL, 74029279521829LL);
  t.b[4] = Q(1335994250573LL, 5691609445217LL);
  t.b[5] = Q(2273837961795LL, 8368240463276LL);
  t.b[6] = Q(247, 2000);
  t.bhat[2] = Q(4469248916618LL, 8635866897933LL);
  t.bhat[3] = Q(-621260224600LL, 4094290005349LL);
  t.bhat[4] = Q(696572312987LL, 2942599194819LL);
  t.bhat[5] = Q(1532940081127LL, 5565293938103LL);
  t.bhat[6] = Q(2441, 20000);
}

ButcherTable ark437_erk() {
  ButcherTable t = make(13, "ARK437L2SA_ERK_7_3_4", 7, 4, 3);
  ark437_common(t);
  t.A[1][0] = Q(247, 1000);
  t.A[2][0] = Q(247, 4000);
  t.A[2][1] = Q(2694949928731LL, 7487940209513LL);
  t.A[3][0] = Q(464650059369LL, 8764239774964LL);
  t.A[3][1] = Q(878889893998LL, 2444806327765LL);
  t.A[3][2] = Q(-952945855348LL, 12294611323341LL);
  t.A[4][0] = Q(476636172619LL, 8159180917465LL);
  t.A[4][1] = Q(-1271469283451LL, 7793814740893LL);
  t.A[4][2] = Q(-859560642026LL, 4356155882851LL);
  t.A[4][3] = Q(1723805262919LL, 4571918432560LL);
  t.A[5][0] = Q(6338158500785LL, 11769362343261LL);
  t.A[5][1] = Q(-4970555480458LL, 10924838743837LL);
  t.A[5][2] = Q(3326578051521LL, 2647936831840LL);
  t.A[5][3] = Q(-880713585975LL, 1841400956686LL);
  t.A[5][4] = Q(-1428733748635LL, 8843423958496LL);
  t.A[6][0] = Q(760814592956LL, 3276306540349LL);
  t.A[6][1] = Q(760814592956LL, 3276306540349LL);
  t.A[6][2] = Q(-47223648122716LL, 6934462133451LL);
  t.A[6][3] = Q(71187472546993LL, 9669769126921LL);
  t.A[6][4] = Q(-13330509492149LL, 9695768672337LL);
  t.A[6][5] = Q(11565764226357LL, 8513123442827LL);
  return t;
}

ButcherTable ark437_dirk() {
  ButcherTable t = make(112, "ARK437L2SA_DIRK_7_3_4", 7, 4, 3);
  ark437_common(t);
  const double g = Q(1235, 10000);
  for (int i = 1; i < 7; ++i) t.A[i][i] = g;
  t.A[1][0] = g;
  t.A[2][0] = t.A[2][1] = Q(624185399699LL, 4186980696204LL);
  t.A[3][0] = t.A[3][1] = Q(1258591069120LL, 10082082980243LL);
  t.A[3][2] = Q(-322722984531LL, 8455138723562LL);
  t.A[4][0] = t.A[4][1] = Q(-436103496990LL, 5971407786587LL);
  t.A[4][2] = Q(-2689175662187LL, 11046760208243LL);
  t.A[4][3] = Q(4431412449334LL, 12995360898505LL);
  t.A[5][0] = t.A[5][1] = Q(-2207373168298LL, 14430576638973LL);
  t.A[5][2] = Q(242511121179LL, 3358618340039LL);
  t.A[5][3] = Q(3145666661981LL, 7780404714551LL);
  t.A[5][4] = Q(5882073923981LL, 14490790706663LL);
  for (int j = 0; j < 6; ++j) t.A[6][j] = t.b[j];
  return t;
}

ButcherTable trbdf2() {
  ButcherTable t = make(102, "TRBDF2_3_3_2", 3, 2, 3);
  const double gd = (2.0 - kRt2) / 2.0, w = kRt2 / 4.0;
  t.c[1] = 2.0 - kRt2; t.c[2] = 1.0;
  t.A[1][0] = gd; t.A[1][1] = gd;
  t.A[2][0] = w; t.A[2][1] = w; t.A[2][2] = gd;
  t.b[0] = w; t.b[1] = w; t.b[2] = gd;
  t.bhat[0] = (1.0 - w) / 3.0; t.bhat[1] = (3.0 * w + 1.0) / 3.0; t.bhat[2] = gd / 3.0;
  return t;
}

#undef Q

struct Registry {
  ButcherTable t[11];
  int n = 0;
  Registry() {
    t[n++] = heun_euler();
    t[n++] = bogacki_shampine();
    t[n++] = ark324_erk();
    t[n++] = zonneveld();
    t[n++] = cash_karp();
    t[n++] = dormand_prince();
    t[n++] = ark437_erk();
    t[n++] = trbdf2();
    t[n++] = ark324_dirk();
    t[n++] = ark437_dirk();
  }
};

const Registry& registry() {
  static const Registry r;
  return r;
}

}  // namespace

const ButcherTable* butcher_table(int id) {
  const Registry& r = registry();
  for (int k = 0; k < r.n; ++k)
    if (r.t[k].id == id) return &r.t[k];
  return nullptr;
}

int erk_default_table(int order) {
  switch (order) {  // ARKODE's default explicit table of each order
    case 2: return 0;
    case 3: return 1;
    case 4: return 3;
    case 5: return 6;
    default: return -1;
  }
}

}  // namespace gbmv

extern "C" int gbmv_butcher_table(int id, gbmv_butcher* out) {
  const gbmv::ButcherTable* t = gbmv::butcher_table(id);
  if (!t || !out) {
    gbmv::set_error("Butcher table %d is not available (explicit 0, 1, 2, 3, 6, 8, 13; "
                    "implicit 102, 104, 112)", id);
    return GBMV_EUNSUPPORTED;
  }
  memset(out, 0, sizeof *out);
  out->id = t->id;
  out->stages = t->s;
  out->q = t->q;
  out->p = t->p;
  strncpy(out->name, t->name, sizeof out->name - 1);
  for (int i = 0; i < t->s; ++i) {
    out->c[i] = t->c[i];
    out->b[i] = t->b[i];
    out->bhat[i] = t->bhat[i];
    for (int j = 0; j < t->s; ++j) out->A[i][j] = t->A[i][j];
  }
  return GBMV_OK;
}

extern "C" int gbmv_erk_default_table(int order) { return gbmv::erk_default_table(order); }
