// Single-rank stand-in for the Boost.MPI calls the reference engine makes:
// every collective copies its input to its output, rank is 0, size is 1.
// Oracle build only.
#pragma once
#include <mpi.h>
#include <algorithm>

namespace boost {
namespace mpl {
struct true_ { static const bool value = true; };
struct false_ { static const bool value = false; };
}  // namespace mpl
namespace mpi {
namespace threading {
enum level { single, funneled, serialized, multiple };
}
class environment {
public:
    environment() {}
    explicit environment(threading::level) {}
};
class communicator {
public:
    int rank() const { return 0; }
    int size() const { return 1; }
    void barrier() const {}
    communicator split(int) const { return communicator(); }
};
template <class T> MPI_Datatype get_mpi_datatype(const T&) { return 0; }
template <class T> struct is_mpi_complex_datatype : mpl::false_ {};
template <class Op, class T> struct is_commutative : mpl::false_ {};

template <class T> void broadcast(const communicator&, T&, int) {}
template <class T, class Op> void all_reduce(const communicator&, const T& in, T& out, Op) { out = in; }
template <class T, class Op> T all_reduce(const communicator&, const T& in, Op) { return in; }
template <class T, class Op> void all_reduce(const communicator&, const T* in, int n, T* out, Op) { std::copy(in, in + n, out); }
template <class T> void all_gather(const communicator&, const T* in, int n, T* out) { std::copy(in, in + n, out); }
template <class T> void all_to_all(const communicator&, const T* in, int n, T* out) { std::copy(in, in + n, out); }
}  // namespace mpi
}  // namespace boost
