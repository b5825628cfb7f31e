// std::vector subclass with the boost::container::vector pieces the reference
// uses: resize(n, default_init). Oracle build only.
#pragma once
#include <cstddef>
#include <memory>
#include <vector>

namespace boost {
namespace container {
struct default_init_t {};
static const default_init_t default_init = default_init_t();

template <class T, class A = std::allocator<T>>
class vector : public std::vector<T, A> {
public:
    using std::vector<T, A>::vector;
    using std::vector<T, A>::resize;
    void resize(std::size_t n, default_init_t) { std::vector<T, A>::resize(n); }
};
}  // namespace container
}  // namespace boost
