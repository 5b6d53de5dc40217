/*
 * Test infrastructure.  The reference GPU program's host main() evaluates
 * WORKER (blockIdx/blockDim/threadIdx) on the host (muca_delta_multigpu.cu:495),
 * which leaves these three symbols undefined in a shared library.  They are
 * defined here so libref_gpuhost.so loads; that main() is never called.
 */
unsigned __device_builtin_variable_blockIdx[3];
unsigned __device_builtin_variable_blockDim[3];
unsigned __device_builtin_variable_threadIdx[3];
