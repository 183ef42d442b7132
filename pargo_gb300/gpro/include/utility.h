// utility.h -- the helpers of the reference's gpro/utility.h that application
// mains use (StringMatch, FileExists, SplitString).
#ifndef PARGO_GPRO_UTILITY_H
#define PARGO_GPRO_UTILITY_H
#include "gpro/gpro.h"
// C++11 spellings the reference's operator headers use
#ifndef OVERRIDE
#define OVERRIDE override
#endif
#ifndef DEFAULT
#define DEFAULT = default
#endif
#ifndef NOEXCEPT
#define NOEXCEPT noexcept
#endif
bool StringMatch(const char* a, const char* b);
bool StringMatch(const string& a, const string& b);
bool FileExists(string const& filename);
vector<string> SplitString(const string& item, char delimiter);
#endif
