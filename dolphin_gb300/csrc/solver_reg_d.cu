// Register-solver instances for K = 46 .. 54 slots (K slots, G threads per pixel
// group); the instances are spread over several translation units so that they compile
// in parallel.
#include "dpl_common.cuh"
#include "pix_args.cuh"
#include "solver.cuh"
#include "solver_reg.cuh"

namespace dpl {

dpl_status launch_solve_reg_d(int K, int G, const PixArgs& a, cudaStream_t s) {
    if (K == 46 && G == 64) return launch_solve_reg_k<46, 64>(a, s);
    if (K == 48 && G == 64) return launch_solve_reg_k<48, 64>(a, s);
    if (K == 50 && G == 64) return launch_solve_reg_k<50, 64>(a, s);
    if (K == 52 && G == 64) return launch_solve_reg_k<52, 64>(a, s);
    if (K == 54 && G == 64) return launch_solve_reg_k<54, 64>(a, s);
    return fail(DPL_ERR_UNSUPPORTED, "register solver: no instance for this slot count and group size");
}

}  // namespace dpl
