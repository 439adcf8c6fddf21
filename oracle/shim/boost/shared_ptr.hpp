// Build shim for compiling the reference library as a CPU oracle:
// boost::shared_ptr is mapped onto std::shared_ptr (same semantics for the
// uses in the reference: construction from new, copy, operator*, ->).
#ifndef ORACLE_SHIM_BOOST_SHARED_PTR_HPP
#define ORACLE_SHIM_BOOST_SHARED_PTR_HPP
#include <memory>
namespace boost { using std::shared_ptr; }
#endif
