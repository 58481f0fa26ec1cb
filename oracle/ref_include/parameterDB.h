/* Test-infrastructure stand-in for the reference's parameterDB: only the
 * lookups that io/parseBodiesFile.cu performs are provided; the body list it
 * fills is a global the harness reads back. */
#pragma once
#include <map>
#include <string>
#include <vector>
class body;
std::vector<body> *ref_body_list();
struct ref_property {
    template <class T> T get() { return reinterpret_cast<T>(ref_body_list()); }
};
struct componentParameter : std::map<std::string, ref_property> {};
struct parameterDB : std::map<std::string, componentParameter> {};
