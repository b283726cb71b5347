/*
 * Stand-in for Boost's <boost/algorithm/string.hpp>, used only to compile the
 * reference's geneticMap.cpp in place (oracle/Makefile -> oracle/_ref).  It
 * provides the two calls that file makes, with Boost's documented meaning:
 * split(out, text, is_any_of(chars)) cuts text at every character of chars
 * and keeps the empty pieces between adjacent separators (Boost's default,
 * token_compress_off).  This file is test infrastructure.
 */
#ifndef GLP_REF_SHIM_BOOST_ALGORITHM_STRING_HPP
#define GLP_REF_SHIM_BOOST_ALGORITHM_STRING_HPP

#include <string>
#include <vector>

namespace boost {

struct glp_any_of {
  std::string chars;
  bool operator()(char ch) const { return chars.find(ch) != std::string::npos; }
};

inline glp_any_of is_any_of(const char *chars) { return glp_any_of{chars}; }

template <class Pred>
std::vector<std::string> &split(std::vector<std::string> &out, const std::string &text,
                                Pred is_separator) {
  out.clear();
  std::string piece;
  for (char ch : text) {
    if (is_separator(ch)) {
      out.push_back(piece);
      piece.clear();
    } else {
      piece.push_back(ch);
    }
  }
  out.push_back(piece);
  return out;
}

}  // namespace boost

#endif
