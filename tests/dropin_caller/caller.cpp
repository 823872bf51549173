// A caller of the drop-in shim written the way the reference's driver calls
// its entry point (LiborMarketModel/main.cpp:65-86): z holds NMAT*numPaths
// normals, liborSwaptionGreeks refills it and returns the value and the
// last delta. Prints them, and z, as one JSON object on stdout.
#include "liborSwaptionGreeks.hpp"

#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char **argv)
{
    const int num_paths = argc > 1 ? std::atoi(argv[1]) : 4096;
    const int nmat = 40;
    std::vector<REAL> z((size_t)nmat * num_paths, (REAL)-7);
    REAL v = 0, lb = 0;
    liborSwaptionGreeks(z.data(), nmat * num_paths, (REAL)0, (REAL)1, 1234, &v, &lb, num_paths);
    std::printf("{\"value\": %.17g, \"delta\": %.17g, \"z\": [", (double)v, (double)lb);
    for (size_t i = 0; i < z.size(); ++i) std::printf(i ? ", %.17g" : "%.17g", (double)z[i]);
    std::printf("]}\n");
    return 0;
}
