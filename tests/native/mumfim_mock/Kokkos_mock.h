// Stand-in for the few Kokkos declarations the integration shim uses: a
// DualView whose host view is a row-major array, sync / modify as no-ops.
// Test infrastructure only; the shim is compiled against it.
#ifndef MFG_TEST_KOKKOS_MOCK_H
#define MFG_TEST_KOKKOS_MOCK_H
#include <cstddef>
#include <memory>
#include <string>
#include <vector>

namespace Kokkos {
struct HostSpace {};
struct DefaultExecutionSpace {};

template <class T> struct RowSize;
template <> struct RowSize<double* [3][3]> { static constexpr size_t value = 9; };
template <> struct RowSize<double* [6][6]> { static constexpr size_t value = 36; };
template <> struct RowSize<double* [6]> { static constexpr size_t value = 6; };
template <> struct RowSize<double* [3]> { static constexpr size_t value = 3; };

template <class DataType, class Space>
class DualView {
 public:
  struct HostView {
    std::shared_ptr<std::vector<double>> buf;
    double* data() const { return buf->data(); }
  };
  HostView h_view;
  DualView() : rows_(0) { h_view.buf = std::make_shared<std::vector<double>>(); }
  DualView(const std::string&, size_t rows) : rows_(rows) {
    h_view.buf = std::make_shared<std::vector<double>>(rows * RowSize<DataType>::value, 0.0);
  }
  size_t extent(int dim) const { return dim == 0 ? rows_ : RowSize<DataType>::value; }
  template <class S> void sync() {}
  template <class S> void modify() { ++modified; }
  int modified = 0;

 private:
  size_t rows_;
};
}  // namespace Kokkos
#endif
