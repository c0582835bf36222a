// AADriskMulti (main.h:269-312, mcBase.h:775-989): one adjoint per payoff.
//
// The reference propagates an nPay-wide adjoint vector through every tape node.  Here each
// payoff's adjoint is a separate reverse sweep over the same paths (same random numbers),
// which yields the exact per-payoff path averages.
#include <vector>

#include "engine.h"

namespace cf {

int Context::riskMulti(Plan& plan, const cf_num_param& num, double* values, double* risks)
{
    std::vector<double> w(plan.nPay, 0.0), r(plan.nParam);
    for (int k = 0; k < plan.nPay; ++k)
    {
        std::fill(w.begin(), w.end(), 0.0);
        w[k] = 1.0;
        int rc = enqueue(plan, num, true, w.data());
        if (rc) return rc;
        rc = fetch(k == 0 ? values : nullptr, nullptr, nullptr, r.data());
        if (rc) return rc;
        for (int j = 0; j < plan.nParam; ++j) risks[size_t(j) * plan.nPay + k] = r[j];
    }
    launches = plan.nPay;
    return CF_OK;
}

}  // namespace cf
