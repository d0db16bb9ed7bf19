// Oracle build shim (test infrastructure only).
// The reference's common/type_processing.hpp:7,14-25 needs only the NAMES of
// three boost::multiprecision types in an NDEBUG build; int256 is used only as
// CompType<int128>, which is never instantiated for capacity types <= int64.
#ifndef LF_ORACLE_BOOST_SHIM_HPP
#define LF_ORACLE_BOOST_SHIM_HPP
namespace boost { namespace multiprecision {
typedef __int128 int128_t;
struct int256_t {};
struct checked_int256_t {};
} }
#endif
