// Mixed-precision form of the PM step (FP32 cell-relative particles, FP32
// deposit and V-cycles inside FP64 defect correction).
#include "pm_common.cuh"

namespace nyxpm {

static nyxpm_status not_built(Ctx& c)
{
    c.err = "mixed-precision form not available";
    return NYXPM_INVALID_ARG;
}

nyxpm_status mixed_unpack(Ctx& c, Box&, const double*, const double*, const double*) { return not_built(c); }
nyxpm_status mixed_pack(Ctx& c, Box&, double*, double*) { return not_built(c); }
nyxpm_status mixed_sort(Ctx& c, Box&) { return not_built(c); }
nyxpm_status mixed_deposit(Ctx& c, Box&) { return not_built(c); }
nyxpm_status mixed_kick(Ctx& c, Box&, double, double, double, int) { return not_built(c); }
nyxpm_status mixed_solve(Ctx& c, Box&, nyxpm_solve_info*) { return not_built(c); }

}  // namespace nyxpm
