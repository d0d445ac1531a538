// Compile-and-run check of include/facetcu.hpp without a GPU: the wrapper
// maps C ABI statuses onto the reference's exception classes.
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "facetcu.hpp"

int main()
{
    const std::vector<facetcu::Direction> dirs = {{0.0f, 1.0f, 0.0f}};
    int checks = 0;
    {
        facetcu::FacetrtCuda model;
        try {
            model.buildVisibilityGraph(dirs);  // before initialize(): logic_error
        } catch (const std::logic_error&) {
            ++checks;
        }
        facetcu::Config config{};
        config.rasterWidth = 0;
        try {
            model.initialize(config);  // invalid raster: invalid_argument
        } catch (const std::invalid_argument&) {
            ++checks;
        }
        facetcu_direction d[40];
        facetcu_hemisphere_directions(40, d);
        if (d[0].y == 0.0125f) ++checks;
    }
    std::printf("%d\n", checks);
    return checks == 3 ? 0 : 1;
}
