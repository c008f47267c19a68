// ref_main_shim.cu -- compiles the reference's src/main.cu where it lies (with
// the Eigen stand-in on the include path) and exposes, with C linkage, the
// reference's own host decoder for tests.  Built by oracle/Makefile into
// oracle/_ref/; the same translation unit compiled with -cubin gives the
// reference's kernels (discrete_solve, eigensetup, modalsetup) for sm_103a.
#include "main.cu"

extern "C" {
// Runs the reference's decode_instructions (src/main.cu:317-337) with
// n_params / BASE_PARAMS set as load_config + upload_plant would set them.
// Returns 0, or 1 with the exception text in err.  out: count x 6 ints/floats
// laid out as the reference's Instruction struct.
int ref_decode(const int* info, int dim, int count, const float* base_params, int n_params, Instruction* out,
               char* err, int errlen) {
    try {
        CFG.n_params = n_params;
        for (int i = 0; i < n_params && i < MAX_PARAMS; i++) BASE_PARAMS_HOST[i] = base_params[i];
        decode_instructions(info, dim, count, out);
        return 0;
    } catch (const std::exception& e) {
        std::snprintf(err, errlen, "%s", e.what());
        return 1;
    }
}
int ref_instruction_size() { return (int)sizeof(Instruction); }
}
