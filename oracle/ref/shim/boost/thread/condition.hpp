/* boost::condition as std::condition_variable_any (used by MULTITHREADING::Sync). */
#pragma once
#include <condition_variable>
namespace boost { typedef std::condition_variable_any condition; }
