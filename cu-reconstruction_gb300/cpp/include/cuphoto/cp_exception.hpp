// Exception type of the reference's host layer (modules/include/cp_exception.hpp:9-22).
#ifndef CUPHOTO_GB300_CP_EXCEPTION_HPP
#define CUPHOTO_GB300_CP_EXCEPTION_HPP

#include <exception>
#include <ostream>
#include <string>

namespace cuphoto {

class CuPhotoException : public std::exception {
public:
    CuPhotoException(const std::string& msg) : message(msg) {}
    CuPhotoException(const char* msg) : message(msg) {}
    const char* what() const noexcept override { return message.c_str(); }
    friend std::ostream& operator<<(std::ostream& os, const CuPhotoException& e) { return os << e.message; }

private:
    std::string message;
};

}  // namespace cuphoto

#endif
