// Register-solver instances for K = 56 .. 64 slots (K slots, G threads per pixel
// group); the instances are spread over several translation units so that they compile
// in parallel.
#include "dpl_common.cuh"
#include "pix_args.cuh"
#include "solver.cuh"
#include "solver_reg.cuh"

namespace dpl {

dpl_status launch_solve_reg_e(int K, int G, const PixArgs& a, cudaStream_t s) {
    if (K == 56 && G == 64) return launch_solve_reg_k<56, 64>(a, s);
    if (K == 58 && G == 64) return launch_solve_reg_k<58, 64>(a, s);
    if (K == 60 && G == 64) return launch_solve_reg_k<60, 64>(a, s);
    if (K == 62 && G == 64) return launch_solve_reg_k<62, 64>(a, s);
    if (K == 64 && G == 64) return launch_solve_reg_k<64, 64>(a, s);
    return fail(DPL_ERR_UNSUPPORTED, "register solver: no instance for this slot count and group size");
}

}  // namespace dpl
