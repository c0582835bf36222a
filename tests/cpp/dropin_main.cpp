// A caller written against the reference's main.h interface, built against cfgpu.hpp
// instead: the store is filled with put*, then value / AADriskOne / AADriskMulti /
// dupireSuperbucket are called with the reference's arguments.  Prints results as JSON.
#include <cmath>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "cfgpu.hpp"

using namespace cfgpu;

int main()
{
    // Dupire 20x10 surface: sigma = 0.15 + 0.10 exp(-t) ln^2(S/100), no noise
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
    putDupire(100.0, spots, times, vols, 0.25, "dupire");
    putBarrier(120.0, 150.0, 3.0, 3.0 / 156.0, 0.01, false, "uoc");
    putBlackScholes(100.0, 0.2, false, 0.02, 0.0, "bs");
    putEuropean(100.0, 1.0, 1.0, "call");
    putEuropeans({1.0, 1.0, 2.0}, {90.0, 110.0, 100.0}, "port");

    NumericalParam num;
    num.useSobol = false;
    num.numPath = 1 << 14;
    const auto v = value("dupire", "uoc", num);
    const auto r = AADriskOne("dupire", "uoc", num, v.identifiers[0]);
    NumericalParam sob;
    sob.useSobol = true;
    sob.numPath = 1 << 14;
    const auto bs = AADriskOne("bs", "call", sob);
    const auto multi = AADriskMulti("dupire", "port", sob);
    bool threw = false;
    try
    {
        value("nope", "uoc", num);
    }
    catch (const std::runtime_error&)
    {
        threw = true;
    }
    const auto dr = dupireAADRisk("dupire", "uoc", {{v.identifiers[0], 1.0}}, num);
    const auto br = bumpRisk("dupire", "uoc", num);
    bool notDupire = false;
    try
    {
        dupireAADRisk("bs", "call", {{"call 1.00 100.00", 1.0}}, sob);
    }
    catch (const std::runtime_error& e)
    {
        notDupire = std::string(e.what()).find("not a Dupire") != std::string::npos;
    }
    // multi-asset: store.h:75-94 and 224-255 with the reference's argument order
    matrix<double> divs(1, 2), correl(2, 2);
    divs[0][0] = 0.02;
    divs[0][1] = 0.0;
    correl[0][0] = correl[1][1] = 1.0;
    correl[0][1] = correl[1][0] = 0.6;
    putDisplaced({"X", "Y"}, {100.0, 100.0}, {0.2, 0.3}, {0.0, -0.05}, 0.02, {0.0, 0.005}, {0.5}, divs, correl, 0.0,
                 "md");
    putAutocall({"X", "Y"}, {100.0, 100.0}, 1.0, 12, 1.02, 0.75, 0.03, 0.02, "ac");
    putBaskets({"X", "Y"}, {0.5, 0.5}, 1.0, {100.0, 108.0}, "bk");
    const auto ac = AADriskOne("md", "ac", sob);
    const auto bk = AADriskMulti("md", "bk", num);
    bool incompatible = false;
    try
    {
        value("dupire", "ac", num);
    }
    catch (const std::runtime_error& e)
    {
        incompatible = std::string(e.what()).find("not compatible") != std::string::npos;
    }
    std::printf("{\"md\": {\"ac_value\": %.17g, \"ac_risks\": [%.17g, %.17g, %.17g], \"ac_nparams\": %zu, "
                "\"ac_label\": \"%s\", \"param12\": \"%s\", \"bk_shape\": [%zu, %zu], \"bk_00\": %.17g, "
                "\"incompatible\": %d},\n",
                ac.riskPayoffValue, ac.risks[0], ac.risks[1], ac.risks[11], ac.risks.size(), ac.payoffIds[0].c_str(),
                ac.paramIds[11].c_str(), bk.risks.rows(), bk.risks.cols(), bk.risks[0][0], incompatible ? 1 : 0);
    std::printf(" \"value\": [%.17g, %.17g], \"risk_value\": %.17g, \"risk0\": %.17g, \"risk5\": %.17g,"
                " \"nparams\": %zu, \"bs\": [%.17g, %.17g, %.17g, %.17g, %.17g], \"multi_shape\": [%zu, %zu],"
                " \"multi00\": %.17g, \"label0\": \"%s\", \"threw\": %d, \"dupire\": [%.17g, %.17g, %.17g],"
                " \"vega_shape\": [%zu, %zu], \"not_dupire\": %d, \"bump_shape\": [%zu, %zu], \"bump50\": %.17g}\n",
                v.values[0], v.values[1], r.riskPayoffValue, r.risks[0], r.risks[5], r.risks.size(),
                bs.riskPayoffValue, bs.risks[0], bs.risks[1], bs.risks[2], bs.risks[3], multi.risks.rows(),
                multi.risks.cols(), multi.risks[0][0], r.payoffIds[0].c_str(), threw ? 1 : 0, dr.value, dr.delta,
                dr.vega[3][4], dr.vega.rows(), dr.vega.cols(), notDupire ? 1 : 0, br.risks.rows(), br.risks.cols(),
                br.risks[50][0]);
    return 0;
}
