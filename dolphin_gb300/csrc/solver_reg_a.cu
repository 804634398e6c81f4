// Register-solver instances for K = 4 .. 16 slots (K slots, G threads per pixel
// group); the instances are spread over several translation units so that they compile
// in parallel.
#include "dpl_common.cuh"
#include "pix_args.cuh"
#include "solver.cuh"
#include "solver_reg.cuh"

namespace dpl {

dpl_status launch_solve_reg_a(int K, int G, const PixArgs& a, cudaStream_t s) {
    if (K == 4 && G == 8) return launch_solve_reg_k<4, 8>(a, s);
    if (K == 4 && G == 16) return launch_solve_reg_k<4, 16>(a, s);
    if (K == 4 && G == 32) return launch_solve_reg_k<4, 32>(a, s);
    if (K == 6 && G == 8) return launch_solve_reg_k<6, 8>(a, s);
    if (K == 6 && G == 16) return launch_solve_reg_k<6, 16>(a, s);
    if (K == 6 && G == 32) return launch_solve_reg_k<6, 32>(a, s);
    if (K == 8 && G == 8) return launch_solve_reg_k<8, 8>(a, s);
    if (K == 8 && G == 16) return launch_solve_reg_k<8, 16>(a, s);
    if (K == 8 && G == 32) return launch_solve_reg_k<8, 32>(a, s);
    if (K == 10 && G == 16) return launch_solve_reg_k<10, 16>(a, s);
    if (K == 10 && G == 32) return launch_solve_reg_k<10, 32>(a, s);
    if (K == 12 && G == 16) return launch_solve_reg_k<12, 16>(a, s);
    if (K == 12 && G == 32) return launch_solve_reg_k<12, 32>(a, s);
    if (K == 14 && G == 16) return launch_solve_reg_k<14, 16>(a, s);
    if (K == 14 && G == 32) return launch_solve_reg_k<14, 32>(a, s);
    if (K == 16 && G == 16) return launch_solve_reg_k<16, 16>(a, s);
    if (K == 16 && G == 32) return launch_solve_reg_k<16, 32>(a, s);
    return fail(DPL_ERR_UNSUPPORTED, "register solver: no instance for this slot count and group size");
}

}  // namespace dpl
