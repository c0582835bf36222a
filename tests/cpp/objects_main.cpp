// A caller written against the reference's object interfaces (mcBase.h: Model<T>, Product<T>,
// RNG and the simulators that take them), built against cfgpu_mc.hpp instead: it constructs a
// Dupire model, an up-and-out call, a Black-Scholes European and a European portfolio, and calls
// mcSimul / mcSimulAAD / mcSimulAADMulti.  Prints the results as JSON.
#include <cmath>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "cfgpu_mc.hpp"

using namespace cfgpu;

static void arr(const char* name, const std::vector<double>& v, bool last = false)
{
    std::printf("\"%s\": [", name);
    for (size_t i = 0; i < v.size(); ++i) std::printf("%s%.17g", i ? ", " : "", v[i]);
    std::printf("]%s\n", last ? "" : ",");
}

int main()
{
    // the same 20x10 surface as the store-API caller
    std::vector<double> spots, times;
    for (int i = 0; i < 20; ++i) spots.push_back(50.0 * std::pow(4.0, i / 19.0));
    for (int j = 0; j < 10; ++j) times.push_back(0.1 + 2.9 * j / 9.0);
    matrix<double> vols(spots.size(), times.size());
    for (size_t i = 0; i < spots.size(); ++i)
        for (size_t j = 0; j < times.size(); ++j)
        {
            const double l = std::log(spots[i] / 100.0);
            vols[i][j] = 0.15 + 0.10 * std::exp(-times[j]) * l * l;
        }
    const size_t n = 4096;

    // mcSimul: the payoff matrix
    Dupire<double> mdl(100.0, spots, times, vols, 0.25);
    UOC<double> prd(120.0, 150.0, 3.0, 3.0 / 156.0, 0.01);
    mrg32k3a rng(12345, 1234);
    const auto paths = mcSimul(prd, mdl, rng, n);

    // mcSimulAAD on Number instances, default aggregator and a weighted one
    Dupire<Number> mdlN(100.0, spots, times, vols, 0.25);
    UOC<Number> prdN(120.0, 150.0, 3.0, 3.0 / 156.0, 0.01);
    const auto aad = mcSimulAAD(prdN, mdlN, rng, n);
    const auto aadW = mcSimulAAD(prdN, mdlN, rng, n, [](const std::vector<Number>& v) { return v[0] + 0.5 * v[1]; });
    bool nonAffine = false;
    try
    {
        mcSimulAAD(prdN, mdlN, rng, n, [](const std::vector<Number>& v) { return v[0] * v[0]; });
    }
    catch (const std::runtime_error&)
    {
        nonAffine = true;
    }

    // Black-Scholes European with Sobol, FP32 path arithmetic
    BlackScholes<Number> bs(100.0, 0.2, false, 0.02, 0.0);
    European<Number> call(100.0, 1.0);
    const auto bsr = mcSimulAAD(call, bs, Sobol(), n, defaultAggregator, CF_FP32);

    // mcSimulAADMulti of a portfolio on the Dupire model
    Europeans<Number> port({{1.0, {90.0, 110.0}}, {2.0, {100.0}}});
    const auto multi = mcSimulAADMulti(port, mdlN, Sobol(), n);

    // the model's parameters are live: a bumped clone prices with its own spot, the original
    // keeps its own
    auto bumped = mdl.clone();
    *bumped->parameters()[0] += 1.0;
    const auto pathsUp = mcSimul(prd, *bumped, rng, n);
    const auto pathsAgain = mcSimul(prd, mdl, rng, n);

    // shapes: timeline, defline, labels, simDim; the RNG's own draws
    Dupire<double> sized(100.0, spots, times, vols, 0.25);
    sized.allocate(prd.timeline(), prd.defline());
    mrg32k3a own(12345, 1234);
    own.init(sized.simDim());
    std::vector<double> g0, g1, u0;
    own.nextG(g0);
    own.nextG(g1);
    own.skipTo(0);
    own.nextU(u0);
    bool incompatible = false;
    try
    {
        struct TwoAssets : public European<double>
        {
            using European<double>::European;
            const std::vector<std::string>& assetNames() const override
            {
                static const std::vector<std::string> a = {"X", "Y"};
                return a;
            }
        };
        mcSimul(TwoAssets(100.0, 1.0), mdl, rng, 16);
    }
    catch (const std::runtime_error&)
    {
        incompatible = true;
    }

    std::printf("{\n");
    std::printf("\"n\": %zu, \"npay\": %zu,\n", paths.size(), paths[0].size());
    arr("path0", paths[0]);
    arr("path1", paths[1]);
    arr("path_last", paths[n - 1]);
    double m0 = 0, m0up = 0, m0again = 0;
    for (size_t i = 0; i < n; ++i)
    {
        m0 += paths[i][0];
        m0up += pathsUp[i][0];
        m0again += pathsAgain[i][0];
    }
    std::printf("\"mean0\": %.17g, \"mean0_up\": %.17g, \"mean0_again\": %.17g,\n", m0 / n, m0up / n, m0again / n);
    std::printf("\"aad_nparams\": %zu,\n", aad.risks.size());
    arr("aad_risks", {aad.risks[0], aad.risks[5], aad.risks[1 + 3 * 10 + 4]});
    arr("aad_aggregated", {aad.aggregated[0], aad.aggregated[1], aad.aggregated[n - 1]});
    arr("aadw_risks", {aadW.risks[0], aadW.risks[5], aadW.risks[1 + 3 * 10 + 4]});
    arr("aadw_aggregated", {aadW.aggregated[0], aadW.aggregated[1]});
    std::printf("\"non_affine_threw\": %d,\n", nonAffine ? 1 : 0);
    arr("bs_risks", bsr.risks);
    std::printf("\"multi_shape\": [%zu, %zu],\n", multi.risks.rows(), multi.risks.cols());
    arr("multi_risks", {multi.risks[0][0], multi.risks[0][2], multi.risks[1 + 4 * 10 + 2][1]});
    arr("multi_path0", multi.payoffs[0]);
    arr("timeline", prd.timeline());
    std::printf("\"defline_n\": %zu, \"defline_num_last\": %d, \"defline_num_first\": %d,\n", prd.defline().size(),
                prd.defline().back().numeraire ? 1 : 0, prd.defline().front().numeraire ? 1 : 0);
    std::printf("\"label0\": \"%s\", \"param5\": \"%s\", \"simdim\": %zu,\n", prd.payoffLabels()[0].c_str(),
                mdl.parameterLabels()[5].c_str(), sized.simDim());
    arr("g0", {g0[0], g0[1], g0[155]});
    arr("g1", {g1[0], g1[1], g1[155]});
    arr("u0", {u0[0], u0[1]});
    std::printf("\"incompatible\": %d\n", incompatible ? 1 : 0);
    std::printf("}\n");
    return 0;
}
