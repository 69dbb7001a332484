/**
 * Runs the host layer's dynamic-time-warping regression test (SPH::testDTWRegression of
 * sphinxsys_gb300/host/sph_solver_cuda.h) on a series read from a text file: one line per
 * snapshot, one value per observation.  Exit status 0 when the series passes against the
 * stored runs of the input folder, 1 when it does not, 2 on a usage error.
 *
 * usage: dtw_regression_check <input_folder> <identifier> <quantity> <series_file>
 */
#include <fstream>
#include <sstream>

#define SPHX_DIMENSION 2
#include "sphinxsys_cuda.h"

int main(int ac, char *av[])
{
    if (ac != 5)
        return 2;
    std::ifstream in(av[4]);
    std::vector<std::vector<SPH::Real>> snapshots;
    for (std::string line; std::getline(in, line);)
    {
        std::stringstream ls(line);
        std::vector<SPH::Real> row;
        for (SPH::Real v; ls >> v;)
            row.push_back(v);
        if (!row.empty())
            snapshots.push_back(row);
    }
    return SPH::testDTWRegression(av[1], av[2], av[3], snapshots) ? 0 : 1;
}
