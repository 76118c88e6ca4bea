// sbp_ops.h -- host-side coefficient tables of the central SBP operators.
// The numbers define the operators and therefore equal the reference's:
// D1 interior stencils and left closure blocks (code/include/sbpops/D1_central.h:243-273)
// and the inverse closure quadrature (code/include/sbpops/HI_central.h:128-147).
// The host scales them by -h^-1 (and the advection speed) before launch.
#pragma once

namespace sbp {
namespace ops {

struct Operator {
  int order, width, cls_sz, cls_width;
  double interior[7];
  double closure[6][9];
  double hinv0;  // closure_invquad[0]
};

inline const Operator& get(int order) {
  static const Operator o2 = {2, 3, 1, 2, {-1. / 2, 0, 1. / 2}, {{-1., 1}}, 2.};
  static const Operator o4 = {4, 5, 4, 6,
                              {1. / 12, -2. / 3, 0., 2. / 3, -1. / 12},
                              {{-24. / 17, 59. / 34, -4. / 17, -3. / 34, 0, 0},
                               {-1. / 2, 0, 1. / 2, 0, 0, 0},
                               {4. / 43, -59. / 86, 0, 59. / 86, -4. / 43, 0},
                               {3. / 98, 0, -59. / 98, 0, 32. / 49, -4. / 49}},
                              48. / 17};
  static const Operator o6 = {
      6, 7, 6, 9,
      {-1. / 60, 3. / 20, -3. / 4, 0, 3. / 4, -3. / 20, 1. / 60},
      {{-21600. / 13649, 104009. / 54596, 30443. / 81894, -33311. / 27298, 16863. / 27298, -15025. / 163788, 0, 0, 0},
       {-104009. / 240260, 0, -311. / 72078, 20229. / 24026, -24337. / 48052, 36661. / 360390, 0, 0, 0},
       {-30443. / 162660, 311. / 32532, 0, -11155. / 16266, 41287. / 32532, -21999. / 54220, 0, 0, 0},
       {33311. / 107180, -20229. / 21436, 485. / 1398, 0, 4147. / 21436, 25427. / 321540, 72. / 5359, 0, 0},
       {-16863. / 78770, 24337. / 31508, -41287. / 47262, -4147. / 15754, 0, 342523. / 472620, -1296. / 7877,
        144. / 7877, 0},
       {15025. / 525612, -36661. / 262806, 21999. / 87602, -25427. / 262806, -342523. / 525612, 0, 32400. / 43801,
        -6480. / 43801, 720. / 43801}},
      43200. / 13649};
  return order == 2 ? o2 : (order == 4 ? o4 : o6);
}

// Smallest grid (points per direction) the library accepts for an order:
// every closure row must read inside the grid (N >= closure width) and the
// left and right closure regions must not overlap (N >= 2 * closure size).
inline long long min_points(int order) { return order == 2 ? 3 : (order == 4 ? 8 : 12); }

}  // namespace ops
}  // namespace sbp
