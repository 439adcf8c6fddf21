// Build shim: boost::noncopyable for the reference's Element base class.
#ifndef ORACLE_SHIM_BOOST_UTILITY_HPP
#define ORACLE_SHIM_BOOST_UTILITY_HPP
namespace boost {
class noncopyable {
 protected:
  noncopyable() {}
  ~noncopyable() {}
 private:
  noncopyable(const noncopyable&);
  noncopyable& operator=(const noncopyable&);
};
}  // namespace boost
#endif
