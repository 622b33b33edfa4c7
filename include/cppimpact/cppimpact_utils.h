// cppimpact_utils.h -- drop-in for include/cppimpact_utils.h.
#pragma once
#include <cstdio>
#include <map>
#include <string>

template <typename T>
void array_to_txt(std::string txt_path, const T* array, int size) {
  std::FILE* fp = std::fopen(txt_path.c_str(), "w");
  if (!fp) {
    std::fprintf(stderr, "Cannot write to %s\n", txt_path.c_str());
    return;
  }
  for (int i = 0; i < size; i++) std::fprintf(fp, "%.16e\n", (double)array[i]);
  std::fclose(fp);
}

// key=value command-line pairs (the reference's parser discards them; these are kept).
class ArgParser {
 public:
  ArgParser(int argc, char* argv[]) {
    for (int i = 1; i < argc; i++) {
      const std::string e(argv[i]);
      const size_t p = e.find('=');
      if (p != std::string::npos) keyvals[e.substr(0, p)] = e.substr(p + 1);
    }
  }
  std::string get(const std::string& k, const std::string& dflt = "") const {
    auto it = keyvals.find(k);
    return it == keyvals.end() ? dflt : it->second;
  }

 private:
  std::map<std::string, std::string> keyvals;
};
