/* stand-in for boost::typeindex (used only in an error message) */
#pragma once
#include <string>
namespace boost { namespace typeindex {
struct gv_type_name { std::string pretty_name() const { return "T"; } };
template <class T> gv_type_name type_id() { return gv_type_name(); }
} }
