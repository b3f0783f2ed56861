/* Headless stand-in for GLFW: the MPM core includes it through mesh.hpp but
 * calls nothing from it. */
#pragma once
inline double glfwGetTime() { return 0.0; }
