/*
 * Single-rank stand-in for the MPI C++ bindings that the reference CPU
 * programs (produce.cpp, muca_mag.cpp) include.  Test infrastructure only:
 * it lets those programs be compiled from their own sources into oracle/_ref
 * on a machine without MPI.  With one rank, Bcast is a no-op and a SUM
 * Reduce copies the send buffer into the receive buffer.
 */
#ifndef ORACLE_MPI_SHIM_H
#define ORACLE_MPI_SHIM_H
#include <cstring>
#include <cstddef>
namespace MPI {
struct Datatype { std::size_t size; };
struct Op { int id; };
static const Datatype DOUBLE = {sizeof(double)};
static const Datatype INT = {sizeof(int)};
static const Datatype UNSIGNED_LONG = {sizeof(unsigned long)};
static const Datatype UNSIGNED_LONG_LONG = {sizeof(unsigned long long)};
static const Op SUM = {0};
struct Intracomm {
    int Get_rank() const { return 0; }
    int Get_size() const { return 1; }
    void Barrier() const {}
    void Bcast(void *, int, const Datatype &, int) const {}
    void Reduce(const void *s, void *r, int n, const Datatype &t, const Op &, int) const {
        if (s != r) std::memcpy(r, s, (std::size_t)n * t.size);
    }
};
static Intracomm COMM_WORLD;
inline void Init() {}
inline void Finalize() {}
}  // namespace MPI
#endif
