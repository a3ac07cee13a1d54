// Debug.hpp — logging: log() is compiled out unless DEBUG_MODE, print() always writes with a
// "[partition]" prefix (the reference's include/Debug.hpp behaviour).
#ifndef DEBUG_HPP
#define DEBUG_HPP

#include <iostream>
#include <string>

#include "NetworkInterface.hpp"

class Debug {
 private:
  static Debug* instance;
  Debug() {}
  template <typename T>
  void rec_log(T t) {
    std::cout << t << std::endl;
  }
  template <typename T, typename... Args>
  void rec_log(T t, Args... args) {
    std::cout << t;
    rec_log(args...);
  }

 public:
  static Debug* get_instance();
  template <typename... Args>
  void log(Args... args) {
#ifdef DEBUG_MODE
    std::cout << "[0] ";
    rec_log(args...);
#endif
  }
  template <typename... Args>
  void print(Args... args) {
    std::cout << "[0] ";
    rec_log(args...);
  }
  void enter_function(std::string func_name);
  void leave_function(std::string func_name);
};

#endif
