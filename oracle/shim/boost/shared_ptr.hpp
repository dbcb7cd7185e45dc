/* Minimal stand-in for boost/shared_ptr.hpp used only to compile the reference
 * CPU path for the oracle: the reference uses nothing of Boost but shared_ptr
 * (libs/stemtypes_fftw3.h:24, libs/imagelib_fftw3.h:7). */
#ifndef QS_SHIM_BOOST_SHARED_PTR_HPP
#define QS_SHIM_BOOST_SHARED_PTR_HPP
#include <memory>
namespace boost { using std::shared_ptr; }
#endif
