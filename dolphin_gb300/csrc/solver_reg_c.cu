// Register-solver instances for K = 34 .. 44 slots (K slots, G threads per pixel
// group); the instances are spread over several translation units so that they compile
// in parallel.
#include "dpl_common.cuh"
#include "pix_args.cuh"
#include "solver.cuh"
#include "solver_reg.cuh"

namespace dpl {

dpl_status launch_solve_reg_c(int K, int G, const PixArgs& a, cudaStream_t s) {
    if (K == 34 && G == 64) return launch_solve_reg_k<34, 64>(a, s);
    if (K == 36 && G == 64) return launch_solve_reg_k<36, 64>(a, s);
    if (K == 38 && G == 64) return launch_solve_reg_k<38, 64>(a, s);
    if (K == 40 && G == 64) return launch_solve_reg_k<40, 64>(a, s);
    if (K == 42 && G == 64) return launch_solve_reg_k<42, 64>(a, s);
    if (K == 44 && G == 64) return launch_solve_reg_k<44, 64>(a, s);
    return fail(DPL_ERR_UNSUPPORTED, "register solver: no instance for this slot count and group size");
}

}  // namespace dpl
