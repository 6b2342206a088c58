// Stand-in for mumfim's exception type. Test infrastructure only.
#ifndef MFG_TEST_EXCEPTIONS_H
#define MFG_TEST_EXCEPTIONS_H
#include <stdexcept>
#include <string>
namespace mumfim {
class mumfim_error : public std::logic_error {
 public:
  explicit mumfim_error(const std::string& err) : std::logic_error{err} {}
  explicit mumfim_error(const char* err) : std::logic_error{err} {}
};
}  // namespace mumfim
#endif
