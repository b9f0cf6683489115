// hyc_eos.cuh -- the 17-term equation of state of the reference for sigma
// at 2000 dbar (stmt_fns.h:183-218 coefficients, :249-263 pressure-folded
// coefficients, :496-505 sig; EOS_17T with EOS_SIG2), in the reference's
// operation order.  Built without FMA contraction by its users, sig17 equals
// the reference's sig() bit for bit (one correctly rounded reciprocal and
// square root).  The 17-term form has no inverse (tofsig is "not available",
// stmt_fns.h:530-532), so only temperature-advecting layers can use it.
#pragma once
#include "hyc_device.cuh"

namespace hyc {

// 17-term equation of state, sigma at rpdb = pref*prs2pdb = 2000 dbar
// (stmt_fns.h:183-218: coefficients; :249-263: pressure-folded ones)
namespace eos17 {
constexpr double c001 = 9.9984085444849347e+02, c002 = 7.3471625860981584e+00, c003 = -5.3211231792841769e-02,
                 c004 = 3.6492439109814549e-04, c005 = 2.5880571023991390e+00, c006 = 6.7168282786692355e-03,
                 c007 = 1.9203202055760151e-03, c008 = 1.0000000000000000e+00, c009 = 7.2815210113327091e-03,
                 c010 = -4.4787265461983921e-05, c011 = 3.3851002965802430e-07, c012 = 1.3651202389758572e-10,
                 c013 = 1.7632126669040377e-03, c014 = 8.8066583251206474e-06, c015 = 1.8832689434804897e-10,
                 c016 = 5.7463776745432097e-06, c017 = 1.4716275472242334e-09, c018 = 1.1798263740430364e-02,
                 c019 = 9.8920219266399117e-08, c020 = 4.6996642771754730e-06, c021 = 2.5862187075154352e-08,
                 c022 = 3.2921414007960662e-12, c023 = 6.7103246285651894e-06, c024 = 2.4461698007024582e-17,
                 c025 = 9.1534417604289062e-18;
constexpr double kRpdb = 2000.e4 * 1.e-4;
constexpr double c101 = c001 + (c018 - c021 * kRpdb) * kRpdb, c103 = c003 + (c019 - c022 * kRpdb) * kRpdb,
                 c105 = c005 + c020 * kRpdb, c108 = c008 + c023 * kRpdb,
                 c109 = c009 - c025 * (kRpdb * kRpdb * kRpdb), c111 = c011 - c024 * (kRpdb * kRpdb);
}  // namespace eos17

// sig(t,s) = sig_n*sig_q - 1000, sig_q = 1/sig_d (stmt_fns.h:497-505)
__device__ __forceinline__ double sig17(double t, double s) {
  using namespace eos17;
  const double sn = c101 + t * (c002 + t * (c103 + t * c004)) + s * (c105 - t * c006 + s * c007);
  const double sd = c108 + t * (c109 + t * (c010 + t * (c111 + t * c012))) +
                    s * (c013 - t * (c014 + t * t * c015) + sqrt(pos0(s)) * (c016 + t * t * c017));
  const double sq = __drcp_rn(sd);  // aone/sig_d, correctly rounded
  return sn * sq - 1000.0;
}

}  // namespace hyc
