/* SCRIPT_READER.h declares boost::regex members; the oracle build never parses a
   script (ref_driver.cpp fills SCRIPT_BLOCK values directly), so std::regex
   only has to make the declarations compile. */
#pragma once
#include <regex>
namespace boost { typedef std::regex regex; using std::regex_search; typedef std::cmatch cmatch; typedef std::smatch smatch; }
