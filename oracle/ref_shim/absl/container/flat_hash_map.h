// Stand-in (test infrastructure for oracle/_ref): the reference only names this map in a comment.
#pragma once
