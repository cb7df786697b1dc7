// Headless console with the reference's command line
// (FasterCapConsole.cpp:33-132): joins argv and runs the GB300 solve path.
#include <stdio.h>
#include <string>
#include "../../include/fastercap_gb300.h"

int main(int argc, char **argv) {
    std::string cmd;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (a.find(' ') != std::string::npos) a = "\"" + a + "\"";
        cmd += a;
        cmd += " ";
    }
    return fcg_run_command_line(cmd.c_str());
}
