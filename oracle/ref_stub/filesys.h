/* empty stand-in for a BOINC header */
